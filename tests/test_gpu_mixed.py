"""Mixed spaces on the GPU: MixedDat / MixedMap arguments and mixed (nested
or monolithic) Mats, against the reference tests' values and the oracle."""
import numpy as np
import pytest

import scenarios as S

pytestmark = pytest.mark.gpu

STRATEGIES = ["atomic", "warp", "colour", "shared", "staged"]


@pytest.fixture(params=STRATEGIES)
def strategy(request, gpu_op2):
    from pyop2_gb300.configuration import configuration
    old = configuration["scatter"]
    configuration["scatter"] = request.param
    yield request.param
    configuration["scatter"] = old


@pytest.mark.parametrize("itspace", [False, True])
@pytest.mark.parametrize("sizes", S.SIZES, ids=["core", "owned", "half"])
def test_mixed_non_mixed_dat(gpu_op2, strategy, sizes, itspace):
    S.sc_mixed_non_mixed_dat(gpu_op2, sizes, itspace)


@pytest.mark.parametrize("nest", [True, False])
def test_mixed_mat(gpu_op2, strategy, nest):
    sp, mat = S.sc_mixed_mat(gpu_op2, nest)
    assert sp.shape == (2, 2) and sp.nested == nest
    if nest:
        assert [list(x) for x in sp.nnz] == [[1, 1, 1], [2, 2, 2], [1, 2, 2, 1], [2, 3, 3, 2]]
    else:
        assert list(sp.nnz) == [3, 3, 3, 3, 5, 5, 3]
    # iteration and indexing of blocks (test/unit/test_api.py:1068-1095)
    for i, block in enumerate(sp):
        assert block is sp[i // 2, i % 2] and block is sp[i // 2][i % 2]
    for i, row in enumerate(mat.blocks):
        for j, m in enumerate(row):
            assert m is mat[i, j] and m.sparsity is sp[i, j]


def test_mixed_rhs(gpu_op2, strategy):
    S.sc_mixed_rhs(gpu_op2)


def test_mixed_rhs_vector(gpu_op2, strategy):
    S.sc_mixed_rhs_vector(gpu_op2)


def _csr(m):
    s = m.to_scipy().tocsr()
    s.sort_indices()
    return s


@pytest.mark.parametrize("nest", [True, False])
def test_mixed_p1p0_matches_oracle(gpu_op2, oracle_op2, strategy, nest):
    """7 x 7 mixed element matrices over 2 x 16^2 cells: every block's
    pattern bit-exact, values and the mixed RHS within 1e-12 (relative)."""
    A, b = S.sc_mixed_p1p0(gpu_op2, 16, nest)
    Ao, bo = S.sc_mixed_p1p0(oracle_op2, 16, nest)
    for i in range(2):
        for j in range(2):
            g, o = A[i, j], Ao[i, j]
            rp, ci = g.sparsity.csr()
            assert np.array_equal(rp, o.sparsity.rowptr)
            assert np.array_equal(ci, o.sparsity.colidx)
            sg, so = _csr(g), _csr(o)
            scale = abs(so).max()
            assert abs(sg - so).max() <= 1e-12 * scale
    if nest:
        assert all(np.array_equal(x, y) for x, y in zip(A.sparsity.nnz, Ao.sparsity.nnz))
    else:
        assert np.array_equal(A.sparsity.nnz, Ao.sparsity.nnz)
    for x, y in zip(b.data_ro, bo.data_ro):
        assert np.abs(x - y).max() <= 1e-12 * np.abs(y).max()
    # the whole matrix, assembled from its blocks
    W, Wo = A.to_scipy(), Ao.to_scipy()
    assert W.shape == (A.nrows, A.ncols) == (289 * 2 + 512,) * 2
    assert abs(W - Wo).max() <= 1e-12 * abs(Wo).max()


def test_mixed_mat_mult(gpu_op2):
    """y = A x block by block equals the assembled whole applied to x."""
    op2 = gpu_op2
    A, _ = S.sc_mixed_p1p0(op2, 16, True)
    rng = np.random.default_rng(5)
    ds = A.sparsity.dsets[1]
    x = op2.MixedDat(ds)
    for d in x:
        d.data[:] = rng.uniform(-1, 1, d.data.shape)
    y = op2.MixedDat(A.sparsity.dsets[0])
    A.mult(x, y)
    xv = np.concatenate([d.data_ro.reshape(-1) for d in x])
    ref = A.to_scipy() @ xv
    got = np.concatenate([d.data_ro.reshape(-1) for d in y])
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()
    yt = op2.MixedDat(A.sparsity.dsets[1])
    A.mult(y, yt, transpose=True)
    reft = A.to_scipy().T @ got
    gott = np.concatenate([d.data_ro.reshape(-1) for d in yt])
    assert np.abs(gott - reft).max() <= 1e-12 * np.abs(reft).max()


def test_mixed_min_max_rw(gpu_op2, oracle_op2):
    """MIN, MAX and RW through a MixedMap, component by component as the
    oracle does them."""
    out = []
    for op2 in (gpu_op2, oracle_op2):
        rng = np.random.default_rng(11)
        it = op2.Set(1000)
        a, bset = op2.Set(300), op2.Set(50)
        ma = op2.Map(it, a, 2, rng.integers(0, 300, (1000, 2)).astype(np.int32))
        mb = op2.Map(it, bset, 1, rng.integers(0, 50, (1000, 1)).astype(np.int32))
        mm = op2.MixedMap((ma, mb))
        src = op2.Dat(it, rng.uniform(-5, 5, 1000))
        lo = op2.MixedDat([op2.Dat(a, np.full(300, 100.0)), op2.Dat(bset, np.full(50, 100.0))])
        hi = op2.MixedDat([op2.Dat(a, np.full(300, -100.0)), op2.Dat(bset, np.full(50, -100.0))])
        op2.par_loop(op2.Kernel("""static void mn(double *lo, double *hi, const double *s) {
            for (int i = 0; i < 3; ++i) { lo[i] = lo[i] < s[0] ? lo[i] : s[0];
                                          hi[i] = hi[i] > s[0] ? hi[i] : s[0]; } }""", "mn"),
                     it, lo(op2.MIN, mm), hi(op2.MAX, mm), src(op2.READ))
        out.append([x.copy() for x in lo.data_ro] + [x.copy() for x in hi.data_ro])
    for g, o in zip(*out):
        assert np.array_equal(g, o)


def test_mixed_dat_version_parloop(gpu_op2):
    """test/unit/test_dats.py:238-256."""
    op2 = gpu_op2
    s = op2.Set(5)
    d3 = op2.Dat(s ** 1, data=None, dtype=np.uint32)
    d4 = op2.Dat(s ** 1, data=None, dtype=np.uint32)
    d3d4 = op2.MixedDat([d3, d4])
    assert d3.dat_version == 0 and d4.dat_version == 0 and d3d4.dat_version == 0
    k = op2.Kernel("""static void write(unsigned int* v) { v[0] = 1; v[1] = 2; }""", "write")
    m = op2.Map(s, op2.Set(5), 1, values=[0, 1, 2, 3, 4])
    op2.par_loop(k, s, d3d4(op2.WRITE, op2.MixedMap([m, m])))
    assert d3.dat_version == 1 and d4.dat_version == 1 and d3d4.dat_version == 2
    assert (d3.data_ro == 1).all() and (d4.data_ro == 2).all()


def test_mixed_linalg(gpu_op2):
    """test/unit/test_linalg.py:316-340, plus componentwise arithmetic."""
    op2 = gpu_op2
    s = op2.Set(1)
    md = op2.MixedDat([op2.Dat(s, [3], np.float64), op2.Dat(s, [4], np.float64)])
    assert abs(md.norm - 5) < 1e-12
    md1 = op2.MixedDat([op2.Dat(s, [4], np.float64), op2.Dat(s, [5], np.float64)])
    assert abs(md.inner(md1) - 32) < 1e-12 and abs(md1.inner(md) - 32) < 1e-12
    r = md + md1
    assert r[0].data_ro[0] == 7 and r[1].data_ro[0] == 9
    r = 2.0 * md - md1
    assert r[0].data_ro[0] == 2 and r[1].data_ro[0] == 3
    md += md1
    assert md[0].data_ro[0] == 7 and md[1].data_ro[0] == 9
    md *= 2.0
    assert md[0].data_ro[0] == 14 and md[1].data_ro[0] == 18


def test_mixed_mat_zero_and_state(gpu_op2):
    op2 = gpu_op2
    sp, mat = S.sc_mixed_mat(op2, True)
    assert mat.assembly_state == op2.Mat.ASSEMBLED
    mat.zero()
    assert all(abs(b.to_scipy()).max() == 0 for b in mat if b.sparsity.nblocks)
    with pytest.raises(NotImplementedError):
        mat.zero_rows([0])
    mat[0, 0].zero_rows([1], 3.0)
    assert mat[0, 0].values[1, 1] == 3.0
