"""Configuration 2b: Map -> CSR sparsity and Mat assembly of the P1 tet
Laplacian on the GPU.  The pattern is compared bit for bit with the oracle
(pyop2/sparsity.pyx semantics) at 16^3 x 6 cells; at 128^3 x 6 cells the
pattern is checked through its exact nonzero count and permutation
invariance, and the assembled matrix through SpMV = matrix-free action."""
import numpy as np
import pytest

from pyop2_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def build(op2, n, permute):
    p = W.build_p1_3d(op2, n=n, permute=permute, seed=0)
    sp = op2.Sparsity((p["verts"] ** 1, p["verts"] ** 1), [(p["c2v"], p["c2v"], None)])
    return p, sp


@pytest.mark.parametrize("permute", [False, True])
def test_sparsity_bit_exact_vs_oracle(gpu_op2, oracle_op2, permute):
    p, sp = build(gpu_op2, 16, permute)
    po, spo = build(oracle_op2, 16, permute)
    rp, ci = sp.csr()
    assert np.array_equal(rp, spo.rowptr)
    assert np.array_equal(ci, spo.colidx)
    assert np.array_equal(sp.nnz, spo.nnz)


@pytest.mark.parametrize("permute", [False, True])
def test_assembly_vs_oracle(gpu_op2, oracle_op2, permute):
    p, sp = build(gpu_op2, 12, permute)
    po, spo = build(oracle_op2, 12, permute)
    A = gpu_op2.Mat(sp)
    Ao = oracle_op2.Mat(spo)
    k = gpu_op2.Kernel(W.P1_3D_LAPLACE_MATRIX, "p1_laplace_3d_mat")
    ko = oracle_op2.Kernel(W.P1_3D_LAPLACE_MATRIX, "p1_laplace_3d_mat")
    gpu_op2.par_loop(k, p["cells"], A(gpu_op2.INC, (p["c2v"], p["c2v"])),
                     p["X"](gpu_op2.READ, p["c2v"]))
    oracle_op2.par_loop(ko, po["cells"], Ao(oracle_op2.INC, (po["c2v"], po["c2v"])),
                        po["X"](oracle_op2.READ, po["c2v"]))
    A.assemble()
    v = A.tensor.cpu().numpy()
    vo = Ao.values_bcsr.reshape(-1)
    assert np.max(np.abs(v - vo)) <= 1e-12 * np.max(np.abs(vo))


def test_full_size_pattern_and_spmv(gpu_op2):
    """128^3 x 6 = 12,582,912 tets: nnz = V + 2 E = 31,802,497 (E = 3n(n+1)^2
    axis + 3n^2(n+1) face-diagonal + n^3 body-diagonal edges), identical row
    counts under a vertex permutation, and A x = the matrix-free action."""
    import torch
    op2 = gpu_op2
    n = 128
    p, sp = build(op2, n, False)
    E = 3 * n * (n + 1) ** 2 + 3 * n * n * (n + 1) + n ** 3
    assert sp.nblocks == (n + 1) ** 3 + 2 * E == 31802497
    A = op2.Mat(sp)
    op2.par_loop(op2.Kernel(W.P1_3D_LAPLACE_MATRIX, "p1_laplace_3d_mat"), p["cells"],
                 A(op2.INC, (p["c2v"], p["c2v"])), p["X"](op2.READ, p["c2v"]))
    A.assemble()
    y_mat = op2.Dat(p["verts"])
    A.mult(p["x"], y_mat)
    p["run"]()          # matrix-free y += K x into the zero y
    a, b = y_mat.data_ro, p["y"].data_ro
    assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
    counts = np.diff(sp.csr()[0])
    del A
    # permutation invariance of the pattern
    from pyop2_gb300 import meshes
    _, cells_p = meshes.unit_cube_tets(n, permute=True, seed=0)
    _, cells_l = meshes.unit_cube_tets(n, permute=False, seed=0)
    pp, spp = build(op2, n, True)
    cp = np.diff(spp.csr()[0])
    # vertex v of the lexicographic mesh is vertex perm[v] of the permuted one
    perm = np.empty(cells_l.max() + 1, dtype=np.int64)
    perm[cells_l.ravel()] = cells_p.ravel()
    assert np.array_equal(cp[perm], counts)
