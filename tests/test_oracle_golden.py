"""The oracle against the reference unit tests' expected values (CPU).

Each scenario in scenarios.py asserts the values the corresponding reference
test asserts; running them on the oracle pins the oracle before it is used to
check the GPU path."""
import numpy as np
import pytest

import scenarios as S


ALL_SIMPLE = [S.sc_indirect_wo, S.sc_indirect_rw, S.sc_indirect_inc, S.sc_indirect_max,
              S.sc_indirect_min, S.sc_global_read, S.sc_global_inc, S.sc_2d_dat]
SIZED = [S.sc_gr_direct_typed, S.sc_gr_read_and_inc, S.sc_gr_minmax, S.sc_gr_mixed_types]
UNSIZED = [S.sc_2d_map, S.sc_itspace_sum_nodes_to_edges, S.sc_vm_read_1d, S.sc_vm_write_1d,
           S.sc_vm_inc_1d, S.sc_vm_read_2d, S.sc_vm_write_2d, S.sc_vm_inc_2d, S.sc_direct,
           S.sc_permuted_map, S.sc_permuted_map_both, S.sc_subset_direct, S.sc_subset_indirect,
           S.sc_extrusion_volume, S.sc_extrusion_direct_inc, S.sc_extrusion_layer_arg,
           S.sc_extrusion_fields,
           S.sc_extrusion_write_coords, S.sc_mass_matrix, S.sc_rhs, S.sc_set_matrix,
           S.sc_vector_mass_matrix, S.sc_sparsity_nnz, S.sc_sparsity_blockwise]


@pytest.mark.parametrize("sizes", S.SIZES, ids=["core", "owned", "half"])
@pytest.mark.parametrize("sc", ALL_SIMPLE + SIZED, ids=lambda f: f.__name__)
def test_oracle_sized(oracle_op2, sc, sizes):
    sc(oracle_op2, sizes)


@pytest.mark.parametrize("sc", UNSIZED, ids=lambda f: f.__name__)
def test_oracle_unsized(oracle_op2, sc):
    sc(oracle_op2)


@pytest.mark.parametrize("permuted", [False, True])
def test_oracle_composed_two(oracle_op2, permuted):
    S.sc_composed_two_maps(oracle_op2, permuted)


@pytest.mark.parametrize("nested", ["none", "first", "last"])
@pytest.mark.parametrize("subset", [False, True])
def test_oracle_composed_three(oracle_op2, nested, subset):
    S.sc_composed_three_maps(oracle_op2, nested, subset)


def test_oracle_extruded_sparsity_rows(oracle_op2):
    """Prism pattern: every row of the 11-layer column couples to the rows of
    the same and the neighbouring level of the nodes it shares cells with."""
    nnz = S.sc_extruded_sparsity(oracle_op2)
    assert nnz.shape == (44,)
    # node 0 (column 0) lies only in element 0: 3 base nodes x (1 or 2 levels)
    assert nnz[0] == 6 and nnz[10] == 6 and nnz[5] == 9


@pytest.mark.parametrize("variable", [False, True])
@pytest.mark.parametrize("subset", [False, True])
def test_oracle_composed_map_extrusion(oracle_op2, variable, subset):
    S.sc_composed_map_extrusion(oracle_op2, variable, subset)
