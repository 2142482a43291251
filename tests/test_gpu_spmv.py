"""Mat.mult (y = A x and y = A^T x) on assembled block-CSR matrices of every
block shape up to 4x4 (each has its own lane kernel) and of shapes beyond
(5x2, 1x6: the tiled kernel), against scipy's product of the same assembled
matrix."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SHAPES = [(1, 1), (2, 2), (3, 3), (2, 3), (1, 2), (4, 4)]
# every block shape up to 4 x 4 has a lane kernel; 5 x 2 and 1 x 6 do not
ALL_SHAPES = [(r, c) for r in range(1, 5) for c in range(1, 5)] + [(5, 2), (1, 6)]


def _assembled(op2, r, c, seed):
    rng = np.random.default_rng(seed)
    ncell, nrow, ncol, ar, ac = 600, 257, 193, 3, 4
    cells = op2.Set(ncell)
    rows = op2.Set(nrow)
    cols = op2.Set(ncol)
    # the last 20 rows are never reached: empty block rows
    rmap = op2.Map(cells, rows, ar, rng.integers(0, nrow - 20, (ncell, ar)).astype(np.int32))
    cmap = op2.Map(cells, cols, ac, rng.integers(0, ncol, (ncell, ac)).astype(np.int32))
    sp = op2.Sparsity((rows ** r, cols ** c), [(rmap, cmap, None)])
    A = op2.Mat(sp)
    w = op2.Dat(cells, rng.uniform(0.5, 1.5, ncell))
    code = """
void elem(double A[%(R)d][%(C)d], const double *w) {
  for (int i = 0; i < %(R)d; ++i)
    for (int j = 0; j < %(C)d; ++j)
      A[i][j] += w[0] * (1.0 + i) / (2.0 + j) - 0.25 * (i == j);
}""" % {"R": ar * r, "C": ac * c}
    op2.par_loop(op2.Kernel(code, "elem"), cells, A(op2.INC, (rmap, cmap)), w(op2.READ))
    A.assemble()
    return A, rows ** r, cols ** c, rng


@pytest.mark.parametrize("shape", SHAPES, ids=["%dx%d" % s for s in SHAPES])
def test_mult_matches_scipy(gpu_op2, shape):
    op2 = gpu_op2
    r, c = shape
    A, drows, dcols, rng = _assembled(op2, r, c, seed=11 * r + c)
    S = A.to_scipy().tocsr()
    assert S.shape == (257 * r, 193 * c)
    x = op2.Dat(dcols, rng.uniform(-1, 1, (193, c)) if c > 1 else rng.uniform(-1, 1, 193))
    y = op2.Dat(drows)
    A.mult(x, y)
    ref = S @ x.data_ro.reshape(-1)
    got = y.data_ro.reshape(-1)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    assert np.all(got[-20 * r:] == 0.0)
    # the same product twice is bitwise identical
    y2 = op2.Dat(drows)
    A.mult(x, y2)
    assert np.array_equal(y2.data_ro, y.data_ro)
    # transpose
    xt = op2.Dat(drows, rng.uniform(-1, 1, (257, r)) if r > 1 else rng.uniform(-1, 1, 257))
    yt = op2.Dat(dcols)
    A.mult(xt, yt, transpose=True)
    reft = S.T @ xt.data_ro.reshape(-1)
    assert np.abs(yt.data_ro.reshape(-1) - reft).max() <= 1e-12 * np.abs(reft).max()


@pytest.mark.parametrize("shape", SHAPES, ids=["%dx%d" % s for s in SHAPES])
def test_mult_inf_only_where_referenced(gpu_op2, shape):
    """x's first column block is +inf: a row that stores no block in that
    column stays finite (lanes past the end of a shorter row in the same
    warp must not touch x), and a row that does is non-finite, as in scipy."""
    op2 = gpu_op2
    r, c = shape
    A, drows, dcols, rng = _assembled(op2, r, c, seed=5 * r + c)
    S = A.to_scipy().tocsr()
    xv = rng.uniform(-1, 1, (193, c))
    xv[0, :] = np.inf
    x = op2.Dat(dcols, xv if c > 1 else xv[:, 0])
    y = op2.Dat(drows)
    with np.errstate(invalid="ignore"):
        A.mult(x, y)
        ref = S @ x.data_ro.reshape(-1)
    got = y.data_ro.reshape(-1)
    refers = np.zeros(257 * r, bool)
    refers[np.unique(S[:, :c].tocoo().row)] = True
    assert refers.any() and not refers.all()
    assert np.all(np.isfinite(got[~refers]))
    assert not np.any(np.isfinite(got[refers]))
    fin = ~refers
    assert np.abs(got[fin] - ref[fin]).max() <= 1e-12 * np.abs(ref[fin]).max()


@pytest.mark.parametrize("shape", SHAPES, ids=["%dx%d" % s for s in SHAPES])
def test_to_torch_export(gpu_op2, shape):
    """torch sparse export (CSR for 1x1, BSR otherwise) equals the scipy
    export entry for entry and shares the Mat's device values."""
    import torch
    op2 = gpu_op2
    r, c = shape
    A, drows, dcols, rng = _assembled(op2, r, c, seed=5 * r + c)
    T = A.to_torch()
    assert T.layout == (torch.sparse_csr if (r, c) == (1, 1) else torch.sparse_bsr)
    assert T.shape == (257 * r, 193 * c) and T.is_cuda
    assert np.array_equal(T.to_dense().cpu().numpy(), A.to_scipy().toarray())
    assert T.values().data_ptr() == A.tensor.data_ptr()
    if (r, c) == (1, 1):
        x = op2.Dat(dcols, rng.uniform(-1, 1, 193))
        y = op2.Dat(drows)
        A.mult(x, y)
        ty = (T @ x.tensor.view(-1, 1)).view(-1)
        assert torch.max(torch.abs(ty - y.tensor)).item() <= 1e-12 * torch.max(torch.abs(y.tensor)).item()


def test_to_torch_mixed(gpu_op2):
    import scenarios as S
    A, _ = S.sc_mixed_p1p0(gpu_op2, 8, False)
    T = A.to_torch()
    assert np.array_equal(T.to_dense().cpu().numpy(), A.to_scipy().toarray())


def test_torch_cg_solve_with_exported_matrix(gpu_op2):
    """The exported device matrix drives a torch solver: conjugate gradients
    on the P1 tet Laplacian of an 8^3 x 6 mesh with Dirichlet rows (zero_rows,
    diagonal 1) equals scipy's direct solve of the same assembled matrix."""
    import scipy.sparse.linalg as spla
    import torch
    from pyop2_gb300 import workloads as W
    op2 = gpu_op2
    p = W.build_p1_3d(op2, n=8, seed=1)
    sp = op2.Sparsity((p["verts"] ** 1, p["verts"] ** 1), [(p["c2v"], p["c2v"], None)])
    A = op2.Mat(sp)
    op2.par_loop(op2.Kernel(W.P1_3D_LAPLACE_MATRIX, "p1_laplace_3d_mat"), p["cells"],
                 A(op2.INC, (p["c2v"], p["c2v"])), p["X"](op2.READ, p["c2v"]))
    A.assemble()
    X = p["coords"]
    bnd = np.where(np.any((X < 1e-12) | (X > 1 - 1e-12), axis=1))[0]
    A.zero_rows(bnd, 1.0)
    S = A.to_scipy().tocsr()
    # keep the operator symmetric: zero the Dirichlet columns too (on both)
    keep = np.ones(S.shape[0])
    keep[bnd] = 0.0
    import scipy.sparse as sps
    D = sps.diags(keep)
    S = (D @ S @ D + sps.diags(1.0 - keep)).tocsr()
    rng = np.random.default_rng(2)
    b = rng.uniform(-1, 1, S.shape[0])
    xs = spla.spsolve(S.tocsc(), b)
    T = A.to_torch()
    dev = T.device
    keep_t = torch.as_tensor(keep, device=dev)

    def matvec(v):   # the same symmetrised operator, on the device
        return keep_t * (T @ (keep_t * v).view(-1, 1)).view(-1) + (1.0 - keep_t) * v

    bt = torch.as_tensor(b, device=dev)
    x = torch.zeros_like(bt)
    r = bt - matvec(x)
    pdir = r.clone()
    rr = torch.dot(r, r)
    for _ in range(500):
        Ap = matvec(pdir)
        alpha = rr / torch.dot(pdir, Ap)
        x += alpha * pdir
        r -= alpha * Ap
        rr_new = torch.dot(r, r)
        if rr_new.sqrt().item() <= 1e-13 * np.linalg.norm(b):
            break
        pdir = r + (rr_new / rr) * pdir
        rr = rr_new
    assert np.max(np.abs(x.cpu().numpy() - xs)) <= 1e-10 * np.max(np.abs(xs))


@pytest.mark.parametrize("shape", ALL_SHAPES, ids=["%dx%d" % s for s in ALL_SHAPES])
def test_mult_every_shape_and_unaligned_values(gpu_op2, shape):
    """y = A x for every block shape against scipy, and through the C ABI
    with the block values copied to an array 8 bytes past an aligned
    address (blocks of 16 or 32 bytes are then loaded one double at a time
    instead of as vectors): the same bits.  y = A^T x likewise, to rounding."""
    import ctypes
    import torch
    from pyop2_gb300 import _lib, device
    op2 = gpu_op2
    r, c = shape
    A, drows, dcols, rng = _assembled(op2, r, c, seed=7 * r + c)
    S = A.to_scipy().tocsr()
    x = op2.Dat(dcols, rng.uniform(-1, 1, (193, c)) if c > 1 else rng.uniform(-1, 1, 193))
    y = op2.Dat(drows)
    A.mult(x, y)
    ref = S @ x.data_ro.reshape(-1)
    got = y.data_ro.reshape(-1).copy()
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    vals = A.tensor
    shifted = torch.zeros(vals.numel() + 1, dtype=torch.float64, device=vals.device)
    shifted[1:].copy_(vals)
    b = A._bcsr()
    b.values = shifted[1:].data_ptr()
    assert b.values % 16 == 8
    y2 = op2.Dat(drows)
    _lib.call("op2g_mat_spmv", ctypes.byref(b), x._device_ptr(), y2._device_ptr(), 0,
              device.stream_handle())
    y2.mark_device_modified()
    assert np.array_equal(y2.data_ro.reshape(-1), got)
    # y = A^T x, from the aligned and from the shifted values (sums by
    # atomics: equal to rounding)
    xt = op2.Dat(drows, rng.uniform(-1, 1, (257, r)) if r > 1 else rng.uniform(-1, 1, 257))
    reft = S.T @ xt.data_ro.reshape(-1)
    for vals_ptr in (None, shifted[1:].data_ptr()):
        yt = op2.Dat(dcols)
        if vals_ptr is None:
            A.mult(xt, yt, transpose=True)
        else:
            b.values = vals_ptr
            yt.tensor.zero_()
            _lib.call("op2g_mat_spmv", ctypes.byref(b), xt._device_ptr(), yt._device_ptr(), 1,
                      device.stream_handle())
            yt.mark_device_modified()
        assert np.abs(yt.data_ro.reshape(-1) - reft).max() <= 1e-12 * np.abs(reft).max()
