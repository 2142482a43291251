"""test/unit/test_matrices.py on the GPU: sparsity construction rules, Mat
diagonal and row operations, WRITE assembly, nbytes, and the assembly state
machine of nested and monolithic mixed matrices.

Reference tests restated under other names: test_mat_always_has_diagonal_space
-> test_sparsity_has_diagonal_space; test_mat_repeated_set_diagonal ->
test_mat_set_diagonal (set twice); test_zero_matrix and test_solve ->
test_zero_matrix_and_solve; test_zero_rows_subset and test_zero_last_row ->
test_zero_rows.  test_assemble_mat, test_assemble_rhs and test_set_matrix
are scenarios.sc_mass_matrix, sc_rhs and sc_set_matrix (run on the GPU and the
oracle); test_matrices_sparsity_blockwise_specification is
sc_sparsity_blockwise.  The FFC-generated variants (test_assemble_ffc,
test_rhs_ffc, test_rhs_ffc_itspace) assert the same values with other kernel
texts and are not restated."""
import numpy as np
import pytest
from numpy.testing import assert_allclose

import scenarios as S

pytestmark = pytest.mark.gpu


@pytest.fixture
def fx(gpu_op2):
    op2 = gpu_op2
    nodes, elements, dnodes, dvnodes, elem_node, coords = S._mat_fixture(op2)
    mat = op2.Mat(op2.Sparsity((dnodes, dnodes), [(elem_node, elem_node, None)],
                               name="sparsity"), np.float64, "mat")
    return op2, nodes, elements, dnodes, elem_node, coords, mat


@pytest.fixture
def mass_mat(fx):
    op2, nodes, elements, dnodes, elem_node, coords, mat = fx
    mat.zero()
    op2.par_loop(op2.Kernel(S.MASS, "mass"), elements, mat(op2.INC, (elem_node, elem_node)),
                 coords(op2.READ, elem_node))
    mat.assemble()
    return mat


def test_sparsity_null_maps(gpu_op2):
    op2 = gpu_op2
    from pyop2_gb300.exceptions import MapValueError
    s = op2.Set(5)
    with pytest.raises(MapValueError):
        m = op2.Map(s, s, 1)
        op2.Sparsity((s ** 1, s ** 1), [(m, m, None)])


def test_sparsity_has_diagonal_space(gpu_op2):
    op2 = gpu_op2
    s, d, d2 = op2.Set(1), op2.Set(4), op2.Set(4)
    m = op2.Map(s, d, 2, [1, 3])
    m2 = op2.Map(s, d2, 3, [1, 2, 3])
    assert all(op2.Sparsity((d ** 1, d ** 1), [(m, m, None)]).nnz == [1, 2, 1, 2])
    assert all(op2.Sparsity((d ** 1, d2 ** 1), [(m, m2, None)]).nnz == [0, 3, 0, 3])


@pytest.mark.parametrize("mode", ["READ", "RW", "MAX", "MIN"])
def test_invalid_mode(fx, mode):
    op2, nodes, elements, dnodes, elem_node, coords, mat = fx
    from pyop2_gb300.exceptions import ModeValueError
    with pytest.raises(ModeValueError):
        op2.par_loop(op2.Kernel("", "dummy"), elements,
                     mat(getattr(op2, mode), (elem_node, elem_node)))


@pytest.mark.parametrize('n', [1, 2])
def test_mat_set_diagonal(fx, n):
    op2, nodes, elements, dnodes, elem_node, coords, _ = fx
    mat = op2.Mat(op2.Sparsity((nodes ** n, nodes ** n), [(elem_node, elem_node, None)]),
                  np.float64)
    nrows = mat.nblock_rows
    for _ in range(2):                    # repeated setting is idempotent
        mat.set_local_diagonal_entries(list(range(nrows)))
        mat.assemble()
        assert (mat.values == np.identity(nrows * n)).all()


def test_minimal_zero_mat(gpu_op2):
    op2 = gpu_op2
    n = 128
    s = op2.Set(n)
    m = op2.Map(s, s, 1, np.arange(n, dtype=np.uint32))
    mat = op2.Mat(op2.Sparsity((s ** 1, s ** 1), [(m, m, None)]), np.float64)
    op2.par_loop(op2.Kernel("void zero_mat(double local_mat[1][1]) { local_mat[0][0] = 0.0; }",
                            "zero_mat"), s, mat(op2.WRITE, (m, m)))
    mat.assemble()
    assert_allclose(mat.values, np.zeros((n, n)), 1e-12)


def test_zero_matrix_and_solve(fx, mass_mat):
    op2, nodes, elements, dnodes, elem_node, coords, mat = fx
    assert_allclose(mass_mat.values, S.EXPECTED_MASS, 1e-5)
    # solve M x = b for the b assembled from f: x = f
    f = op2.Dat(dnodes, np.asarray([1.0, 2.0, 3.0, 4.0]), np.float64, "f")
    b = op2.Dat(dnodes, np.zeros(4), np.float64, "b")
    op2.par_loop(op2.Kernel(S.RHS, "rhs"), elements, b(op2.INC, elem_node),
                 coords(op2.READ, elem_node), f(op2.READ, elem_node))
    assert_allclose(np.linalg.solve(mass_mat.values, b.data), f.data, 1e-8)
    mass_mat.zero()
    assert_allclose(mass_mat.values, np.zeros((4, 4)), 1e-14)


def test_zero_rhs(fx):
    op2, nodes, elements, dnodes, elem_node, coords, mat = fx
    b = op2.Dat(dnodes, np.ones(4), np.float64, "b")
    op2.par_loop(op2.Kernel("static void zero_dat(double *dat) { *dat = 0.0; }", "zero_dat"),
                 nodes, b(op2.WRITE))
    assert all(b.data == 0)


def test_zero_rows(fx, mass_mat):
    op2, nodes = fx[0], fx[1]
    expected = S.EXPECTED_MASS.copy()
    expected[0] = [12.0, 0.0, 0.0, 0.0]
    mass_mat.zero_rows([0], 12.0)
    assert_allclose(mass_mat.values, expected, 1e-5)
    mass_mat.zero_rows(op2.Subset(nodes, [0]), 12.0)
    assert_allclose(mass_mat.values, expected, 1e-5)
    expected[3] = [0.0, 0.0, 0.0, 4.0]
    mass_mat.zero_rows([3], 4.0)
    assert_allclose(mass_mat.values, expected, 1e-5)


def test_mat_nbytes(fx):
    assert fx[-1].nbytes == 14 * 8


# ---- assembly state machine of mixed matrices
@pytest.fixture(params=[False, True], ids=["Non-nested", "Nested"])
def mmat(request, gpu_op2):
    op2 = gpu_op2
    elem, node, mset, mdat, mmap, rdata = S._mixed_mat_fixture(op2)
    blocks = {(i, j): [(rm, cm, None)] for i, rm in enumerate(mmap) for j, cm in enumerate(mmap)}
    return op2, op2.Mat(op2.Sparsity((mset ** 1, mset ** 1), blocks, nest=request.param))


def test_mat_starts_assembled(mmat):
    op2, mat = mmat
    assert mat.assembly_state is op2.Mat.ASSEMBLED
    assert all(m.assembly_state is op2.Mat.ASSEMBLED for m in mat)


def test_after_set_local_state_is_insert(mmat):
    op2, mat = mmat
    mat[0, 0].set_local_diagonal_entries([0])
    assert mat[0, 0].assembly_state is op2.Mat.INSERT_VALUES
    if not mat.sparsity.nested:
        assert mat.assembly_state is op2.Mat.INSERT_VALUES
    else:
        assert mat[1, 1].assembly_state is op2.Mat.ASSEMBLED


def test_after_addto_state_is_add(mmat):
    op2, mat = mmat
    mat[0, 0].addto_values(0, 0, [1])
    assert mat[0, 0].assembly_state is op2.Mat.ADD_VALUES
    if not mat.sparsity.nested:
        assert mat.assembly_state is op2.Mat.ADD_VALUES
    else:
        assert mat[1, 1].assembly_state is op2.Mat.ASSEMBLED


def test_matblock_assemble_runtimeerror(mmat):
    op2, mat = mmat
    if mat.sparsity.nested:
        return
    with pytest.raises(RuntimeError):
        mat[0, 0].assemble()


def test_mixing_insert_and_add_works(mmat):
    op2, mat = mmat
    mat[0, 0].addto_values(0, 0, [1])
    mat[1, 1].addto_values(1, 1, [3])
    mat[1, 1].set_values(0, 0, [2])
    mat[0, 0].set_values(1, 1, [4])
    mat[1, 1].addto_values(0, 0, [3])
    mat.assemble()
    assert np.allclose(mat[0, 0].values, np.diag([1, 4, 0]))
    assert np.allclose(mat[1, 1].values, np.diag([5, 3, 0, 0]))
    assert np.allclose(mat[0, 1].values, 0) and np.allclose(mat[1, 0].values, 0)


def test_assembly_flushed_between_insert_and_add(mmat):
    import types
    op2, mat = mmat
    flush_counter = [0]

    def make_flush(old_flush):
        def flush(self):
            old_flush()
            flush_counter[0] += 1
        return flush
    mat._flush_assembly = types.MethodType(make_flush(mat._flush_assembly), mat)
    if mat.sparsity.nested:
        for m in mat:
            m._flush_assembly = types.MethodType(make_flush(m._flush_assembly), m)
    mat[0, 0].addto_values(0, 0, [1])
    assert flush_counter[0] == 0
    # the reference inserts at (1, 0) after switching PETSc's new-nonzero
    # errors off; the pattern here is fixed, so an entry inside it is used
    mat[0, 0].set_values(1, 1, [2])
    assert flush_counter[0] == 1
    mat.assemble()
    assert flush_counter[0] == 1
