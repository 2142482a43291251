"""The reference's unit tests, run on the GPU through pyop2_gb300.op2.

Each scenario asserts the reference test's own expected values; INC-carrying
scenarios also run under every conflict strategy (atomics, warp-aggregated
atomics, colouring)."""
import numpy as np
import pytest

import scenarios as S
from test_oracle_golden import ALL_SIMPLE, SIZED, UNSIZED

pytestmark = pytest.mark.gpu

STRATEGIES = ["atomic", "warp", "colour", "shared", "staged"]


@pytest.fixture(params=STRATEGIES)
def strategy(request, gpu_op2):
    from pyop2_gb300.configuration import configuration
    old = configuration["scatter"]
    configuration["scatter"] = request.param
    yield request.param
    configuration["scatter"] = old


@pytest.mark.parametrize("sizes", S.SIZES, ids=["core", "owned", "half"])
@pytest.mark.parametrize("sc", ALL_SIMPLE + SIZED, ids=lambda f: f.__name__)
def test_gpu_sized(gpu_op2, sc, sizes):
    sc(gpu_op2, sizes)


@pytest.mark.parametrize("sc", UNSIZED, ids=lambda f: f.__name__)
def test_gpu_unsized(gpu_op2, strategy, sc):
    if sc is S.sc_extrusion_write_coords:
        sc(gpu_op2, sequential=False)
    else:
        sc(gpu_op2)


@pytest.mark.parametrize("sc", [S.sc_indirect_inc, S.sc_global_inc, S.sc_indirect_min,
                                S.sc_indirect_max], ids=lambda f: f.__name__)
def test_gpu_strategies(gpu_op2, strategy, sc):
    sc(gpu_op2)


@pytest.mark.parametrize("permuted", [False, True])
def test_gpu_composed_two(gpu_op2, permuted):
    S.sc_composed_two_maps(gpu_op2, permuted)


@pytest.mark.parametrize("nested", ["none", "first", "last"])
@pytest.mark.parametrize("subset", [False, True])
def test_gpu_composed_three(gpu_op2, nested, subset):
    S.sc_composed_three_maps(gpu_op2, nested, subset)


def test_gpu_matrix_values_match_oracle(gpu_op2, oracle_op2):
    np.testing.assert_allclose(S.sc_mass_matrix(gpu_op2), S.sc_mass_matrix(oracle_op2),
                               rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(S.sc_vector_mass_matrix(gpu_op2),
                               S.sc_vector_mass_matrix(oracle_op2), rtol=1e-12, atol=1e-15)
    np.testing.assert_allclose(S.sc_rhs(gpu_op2), S.sc_rhs(oracle_op2), rtol=1e-12)


def test_gpu_extruded_sparsity_matches_oracle(gpu_op2, oracle_op2):
    assert np.array_equal(S.sc_extruded_sparsity(gpu_op2), S.sc_extruded_sparsity(oracle_op2))


def test_gpu_extrusion_volume_matches_oracle(gpu_op2, oracle_op2):
    assert abs(S.sc_extrusion_volume(gpu_op2) - S.sc_extrusion_volume(oracle_op2)) <= 1e-12


def test_gpu_zero_rows_and_diagonal(gpu_op2):
    """test/unit/test_matrices.py:582-602, 740-768."""
    op2 = gpu_op2
    nodes, elements, dnodes, dvnodes, elem_node, coords = S._mat_fixture(op2)
    mat = op2.Mat(op2.Sparsity((dnodes, dnodes), [(elem_node, elem_node, None)]))
    op2.par_loop(op2.Kernel(S.MASS, "mass"), elements, mat(op2.INC, (elem_node, elem_node)),
                 coords(op2.READ, elem_node))
    mat.assemble()
    expected = S.EXPECTED_MASS.copy()
    expected[0] = [12.0, 0.0, 0.0, 0.0]
    mat.zero_rows([0], 12.0)
    np.testing.assert_allclose(mat.values, expected, 1e-5)
    expected[3] = [0.0, 0.0, 0.0, 4.0]
    mat.zero_rows(op2.Subset(nodes, [3]), 4.0)
    np.testing.assert_allclose(mat.values, expected, 1e-5)
    for n in (1, 2):
        m2 = op2.Mat(op2.Sparsity((nodes ** n, nodes ** n), [(elem_node, elem_node, None)]))
        m2.set_local_diagonal_entries(list(range(m2.nblock_rows)))
        m2.assemble()
        assert (m2.values == np.identity(4 * n)).all()
    assert mat.nbytes == 14 * 8


def test_gpu_new_nonzero_is_reported(gpu_op2):
    """Inserting outside the pattern raises at assemble() (PETSc's
    NEW_NONZERO_LOCATION_ERR, pyop2/types/mat.py:723-724)."""
    op2 = gpu_op2
    s = op2.Set(2)
    nodes = op2.Set(4)
    m1 = op2.Map(s, nodes, 2, [[0, 1], [2, 3]])
    m2 = op2.Map(s, nodes, 2, [[0, 2], [1, 3]])
    mat = op2.Mat(op2.Sparsity((nodes ** 1, nodes ** 1), [(m1, m1, None), (m2, m2, None)]))
    k = op2.Kernel("static void k(double A[2][2]) { A[0][1] += 1.0; }", "k")
    m3 = op2.Map(s, nodes, 2, [[0, 3], [3, 0]])
    from pyop2_gb300.parloop import MatLegacyArg
    op2.par_loop(k, s, MatLegacyArg(mat, (m3, m3), op2.INC))
    with pytest.raises(RuntimeError):
        mat.assemble()


def test_gpu_addto_and_set_values_state_machine(gpu_op2):
    """test/unit/test_matrices.py:775-862 on a single block: addto/set change
    the assembly state, mixing them works, values land where expected."""
    op2 = gpu_op2
    s = op2.Set(3)
    m = op2.Map(s, s, 1, [0, 1, 2])
    mat = op2.Mat(op2.Sparsity((s ** 1, s ** 1), [(m, m, None)]))
    assert mat.assembly_state is op2.Mat.ASSEMBLED
    mat.addto_values(0, 0, [1])
    assert mat.assembly_state is op2.Mat.ADD_VALUES
    mat.set_values(1, 1, [4])
    assert mat.assembly_state is op2.Mat.INSERT_VALUES
    mat.addto_values(0, 0, [3])
    mat.assemble()
    assert mat.assembly_state is op2.Mat.ASSEMBLED
    assert np.allclose(mat.values, np.diag([4, 4, 0]))
    with pytest.raises(RuntimeError):
        mat.set_values(0, 2, [1])      # outside the (diagonal) pattern
