"""Direct Dat arguments whose rows are a multiple of 16 bytes run through a
wrapper variant that declares each row aligned (so the kernel's accesses to
adjacent components become vector loads and stores) when the Dat's array is
aligned, and through the plain wrapper when it is not.  Both must give the
expected values, including PyOP2's pointer semantics for a direct WRITE
argument: components the kernel does not write keep their values.  Indirect
rows of the same sizes, from aligned and offset arrays, are checked too."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (C type, numpy dtype, dim): 32-byte rows, 16-byte rows, and rows that get
# no alignment hint (24 and 12 bytes)
CASES = [("double", np.float64, 4), ("double", np.float64, 2), ("float", np.float32, 4),
         ("long long", np.int64, 2), ("double", np.float64, 3), ("float", np.float32, 3)]
IDS = ["f64x4", "f64x2", "f32x4", "i64x2", "f64x3", "f32x3"]


def _loop(op2, ctype, dt, dim, out, rw, every):
    """out (direct, dim components) from four gathered vertex values."""
    rng = np.random.default_rng(dim * 7 + len(ctype))
    cells, verts = out.dataset.set, op2.Set(97)
    c2v = op2.Map(cells, verts, 4, rng.integers(0, 97, (cells.size, 4)).astype(np.int32))
    x = op2.Dat(verts, rng.integers(-50, 50, 97).astype(dt), dt)
    op = "+=" if rw else "="
    src = ("static void k(%(T)s *o, const %(T)s *x) {\n"
           "  for (int i = 0; i < %(D)d; i += %(E)d) o[i] %(op)s x[i %% 4] * (%(T)s)(i + 1);\n"
           "}\n") % {"T": ctype, "D": dim, "E": every, "op": op}
    op2.par_loop(op2.Kernel(src, "k"), cells, out(op2.RW if rw else op2.WRITE), x(op2.READ, c2v))
    return c2v.values, x.data_ro


def _expected(init, mv, xv, dim, rw, every):
    want = init.copy()
    for i in range(0, dim, every):
        v = xv[mv[:, i % 4]] * (i + 1)
        want[:, i] = want[:, i] + v if rw else v
    return want


@pytest.mark.parametrize("case", CASES, ids=IDS)
@pytest.mark.parametrize("offset", [0, 1], ids=["aligned", "offset"])
@pytest.mark.parametrize("mode", ["write", "write_every_other", "rw"])
def test_direct_rows(gpu_op2, case, offset, mode):
    import torch
    op2 = gpu_op2
    ctype, dt, dim = case
    rw, every = mode == "rw", (2 if mode == "write_every_other" else 1)
    n = 1000
    cells = op2.Set(n)
    init = (np.arange(n * dim).reshape(n, dim) % 13 - 6).astype(dt)
    tdt = {np.float64: torch.float64, np.float32: torch.float32, np.int64: torch.int64}[dt]
    # the Dat's array starts `offset` elements into a larger allocation
    base = torch.full((n * dim + offset + 8,), -99, dtype=tdt, device="cuda")
    base[offset:offset + n * dim] = torch.from_numpy(init.reshape(-1)).cuda()
    out = op2.Dat.from_tensor(cells ** dim, base[offset:offset + n * dim])
    assert (out.tensor.data_ptr() % 16 == 0) == (offset == 0)
    mv, xv = _loop(op2, ctype, dt, dim, out, rw, every)
    got = out.data_ro.reshape(n, dim)
    assert np.array_equal(got, _expected(init, mv, xv, dim, rw, every))
    # nothing outside the Dat's rows was written
    rest = torch.cat([base[:offset], base[offset + n * dim:]]).cpu().numpy()
    assert np.all(rest == -99)


def test_same_loop_switches_variant(gpu_op2):
    """One built loop launched on an aligned and then on an offset array
    (the pointer is re-read at each launch) gives the same values."""
    import torch
    from pyop2_gb300.parloop import LegacyParloop
    op2 = gpu_op2
    n, dim = 777, 4
    cells, verts = op2.Set(n), op2.Set(50)
    rng = np.random.default_rng(3)
    c2v = op2.Map(cells, verts, 4, rng.integers(0, 50, (n, 4)).astype(np.int32))
    x = op2.Dat(verts, rng.uniform(-1, 1, 50))
    big = torch.zeros(n * dim + 1, dtype=torch.float64, device="cuda")
    out = op2.Dat.from_tensor(cells ** dim, big[:n * dim])
    lp = LegacyParloop(op2.Kernel("static void k(double *o, const double *x) "
                                  "{ for (int i = 0; i < 4; ++i) o[i] = 2.0 * x[i]; }", "k"),
                       cells, out(op2.WRITE), x(op2.READ, c2v))
    lp.compute()
    first = out.data_ro.copy()
    out._rebind(big[1:])
    lp.compute()
    assert np.array_equal(out.data_ro, first)
    assert np.array_equal(first, 2.0 * x.data_ro[c2v.values])


@pytest.mark.parametrize("case", CASES, ids=IDS)
@pytest.mark.parametrize("offset", [0, 1], ids=["aligned", "offset"])
def test_indirect_rows(gpu_op2, case, offset):
    """Indirect rows of 12 to 32 bytes from an aligned and from an offset
    array: gathered (READ) through a map, and read and written back (RW)
    through a bijection."""
    import torch
    op2 = gpu_op2
    ctype, dt, dim = case
    tdt = {np.float64: torch.float64, np.float32: torch.float32, np.int64: torch.int64}[dt]
    n, nv = 500, 120
    rng = np.random.default_rng(dim + offset)
    cells, verts = op2.Set(n), op2.Set(nv)
    c2v = op2.Map(cells, verts, 3, rng.integers(0, nv, (n, 3)).astype(np.int32))
    vals = rng.integers(-9, 10, (nv, dim)).astype(dt)
    base = torch.full((nv * dim + offset + 4,), -99, dtype=tdt, device="cuda")
    base[offset:offset + nv * dim] = torch.from_numpy(vals.reshape(-1)).cuda()
    xv = op2.Dat.from_tensor(verts ** dim, base[offset:offset + nv * dim])
    out = op2.Dat(cells, np.zeros(n, dtype=dt), dt)
    src = ("static void k(%(T)s *o, const %(T)s *x) {\n"
           "  %(T)s s = 0;\n"
           "  for (int i = 0; i < 3; ++i)\n"
           "    for (int j = 0; j < %(D)d; ++j) s += x[i * %(D)d + j] * (%(T)s)(1 + i + 3 * j);\n"
           "  o[0] = s;\n"
           "}\n") % {"T": ctype, "D": dim}
    op2.par_loop(op2.Kernel(src, "k"), cells, out(op2.WRITE), xv(op2.READ, c2v))
    w = np.array([[1 + i + 3 * j for j in range(dim)] for i in range(3)], dtype=dt)
    want = np.einsum("cij,ij->c", vals[c2v.values], w).astype(dt)
    assert np.array_equal(out.data_ro, want)
    # RW through a bijection of the vertices
    bij = op2.Map(verts, verts, 1, rng.permutation(nv).astype(np.int32).reshape(nv, 1))
    rw = ("static void r(%(T)s *y) {\n"
          "  for (int j = 0; j < %(D)d; ++j) y[j] = y[j] * (%(T)s)2 + (%(T)s)j;\n"
          "}\n") % {"T": ctype, "D": dim}
    op2.par_loop(op2.Kernel(rw, "r"), verts, xv(op2.RW, bij))
    assert np.array_equal(xv.data_ro.reshape(nv, dim), vals * 2 + np.arange(dim, dtype=dt))
    rest = torch.cat([base[:offset], base[offset + nv * dim:]]).cpu().numpy()
    assert np.all(rest == -99)
