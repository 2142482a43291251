"""test/unit/test_global_reduction.py on the GPU: READ/INC/MIN/MAX Globals of
every element type through direct loops, repeated and reused loops.

Reference tests restated here, several per function:
test_direct_typed -- test_direct_{min,max}_{uint32,int32,float,double};
test_1d_read -- test_1d_read, test_1d_read_no_init; test_2d_read;
test_1d_inc -- test_1d_inc, test_1d_inc_no_data;
test_1d_min_max -- test_1d_{min,max}_dat_is_{min,max},
test_1d_{min,max}_global_is_{min,max}; test_2d_inc_min_max -- test_2d_inc,
test_2d_{min,max}_dat_is_{min,max}, test_2d_{min,max}_global_is_{min,max};
test_multi_inc -- test_1d_multi_inc_same_global(_reset),
test_1d_multi_inc_diff_global; test_globals_with_different_types;
test_inc_repeated_and_reused_loop -- test_inc_repeated_loop,
test_inc_reused_loop."""
import numpy as np
import pytest
from numpy.testing import assert_allclose

pytestmark = pytest.mark.gpu

NEL = 4096

K1_WRITE = "static void k(unsigned int *x, unsigned int *g) { *x = *g; }"
K1_INC = "static void k(unsigned int *g, unsigned int *x) { *g += *x; }"
K1_MIN = "static void k(unsigned int *g, unsigned int *x) { if (*x < *g) *g = *x; }"
K1_MAX = "static void k(unsigned int *g, unsigned int *x) { if (*x > *g) *g = *x; }"
K2_MIN = """static void k(unsigned int *g, unsigned int *x) {
  if (x[0] < g[0]) g[0] = x[0];
  if (x[1] < g[1]) g[1] = x[1]; }"""
K2_MAX = """static void k(unsigned int *g, unsigned int *x) {
  if (x[0] > g[0]) g[0] = x[0];
  if (x[1] > g[1]) g[1] = x[1]; }"""
K2_WRITE = "static void k(unsigned int *x, unsigned int *g) { *x = g[0] + g[1]; }"
K2_INC = "static void k(unsigned int *g, unsigned int *x) { g[0] += x[0]; g[1] += x[1]; }"


@pytest.fixture(params=[(NEL, NEL, NEL), (0, NEL, NEL), (NEL // 2, NEL, NEL)])
def env(request, gpu_op2):
    op2 = gpu_op2
    s = op2.Set(request.param, 'set')
    dset, dset2 = op2.DataSet(s, 1, 'set'), op2.DataSet(s, 2, 'set2')
    d1 = op2.Dat(dset, np.arange(NEL) + 1, dtype=np.uint32)
    d2 = op2.Dat(dset2, np.arange(2 * NEL) + 1, dtype=np.uint32)
    return op2, s, dset, d1, d2


@pytest.mark.parametrize("dt,ctype,init,fill,acc,expect", [
    (np.uint32, "unsigned int", 8, 12, "MIN", 8),
    (np.int32, "int", 8, -12, "MIN", -12),
    (np.int32, "int", -42, -12, "MAX", -12),
    (np.float32, "float", -.8, -12.0, "MIN", -12.0),
    (np.float32, "float", -42.8, -12.0, "MAX", -12.0),
    (np.float64, "double", -.8, -12.0, "MIN", -12.0),
    (np.float64, "double", -42.8, -12.0, "MAX", -12.0)])
def test_direct_typed(env, dt, ctype, init, fill, acc, expect):
    op2, s, dset, d1, d2 = env
    d = op2.Dat(dset, [fill] * NEL, dt)
    cmp = "<" if acc == "MIN" else ">"
    k = "static void k(%s* g, %s* x) { if ( *x %s *g ) *g = *x; }" % (ctype, ctype, cmp)
    g = op2.Global(1, init, dt, "g")
    op2.par_loop(op2.Kernel(k, "k"), s, g(getattr(op2, acc)), d(op2.READ))
    assert_allclose(g.data[0], expect)


def test_1d_read(env):
    op2, s, dset, d1, d2 = env
    g = op2.Global(1, 1, dtype=np.uint32)
    op2.par_loop(op2.Kernel(K1_WRITE, "k"), s, d1(op2.WRITE), g(op2.READ))
    assert all(d1.data == g.data)
    g = op2.Global(1, dtype=np.uint32)
    d1.data[:] = 100
    op2.par_loop(op2.Kernel(K1_WRITE, "k"), s, d1(op2.WRITE), g(op2.READ))
    assert all(g.data == 0) and all(d1.data == 0)


def test_2d_read(env):
    op2, s, dset, d1, d2 = env
    g = op2.Global(2, (1, 2), dtype=np.uint32)
    op2.par_loop(op2.Kernel(K2_WRITE, "k"), s, d1(op2.WRITE), g(op2.READ))
    assert all(d1.data == g.data.sum())


def test_1d_inc(env):
    op2, s, dset, d1, d2 = env
    for g in (op2.Global(1, 0, dtype=np.uint32), op2.Global(1, dtype=np.uint32)):
        op2.par_loop(op2.Kernel(K1_INC, "k"), s, g(op2.INC), d1(op2.READ))
        assert g.data == d1.data.sum()


def test_1d_min_max(env):
    op2, s, dset, d1, d2 = env
    g = op2.Global(1, d1.data.min() + 1, dtype=np.uint32)
    op2.par_loop(op2.Kernel(K1_MIN, "k"), s, g(op2.MIN), d1(op2.READ))
    assert g.data == d1.data.min()
    g = op2.Global(1, d1.data.max() - 1, dtype=np.uint32)
    op2.par_loop(op2.Kernel(K1_MAX, "k"), s, g(op2.MAX), d1(op2.READ))
    assert g.data == d1.data.max()
    val = d1.data.max() + 1
    g = op2.Global(1, val, dtype=np.uint32)
    op2.par_loop(op2.Kernel(K1_MAX, "k"), s, g(op2.MAX), d1(op2.READ))
    assert g.data == val
    d1.data[:] += 10
    val = d1.data.min() - 1
    g = op2.Global(1, val, dtype=np.uint32)
    op2.par_loop(op2.Kernel(K1_MIN, "k"), s, g(op2.MIN), d1(op2.READ))
    assert g.data == val


def test_2d_inc_min_max(env):
    op2, s, dset, d1, d2 = env
    g = op2.Global(2, (0, 0), dtype=np.uint32)
    op2.par_loop(op2.Kernel(K2_INC, "k"), s, g(op2.INC), d2(op2.READ))
    assert g.data[0] == d2.data[:, 0].sum() and g.data[1] == d2.data[:, 1].sum()
    g = op2.Global(2, (d2.data[:, 0].min() + 1, d2.data[:, 1].min() + 1), dtype=np.uint32)
    op2.par_loop(op2.Kernel(K2_MIN, "k"), s, g(op2.MIN), d2(op2.READ))
    assert g.data[0] == d2.data[:, 0].min() and g.data[1] == d2.data[:, 1].min()
    g = op2.Global(2, (d2.data[:, 0].max() - 1, d2.data[:, 1].max() - 1), dtype=np.uint32)
    op2.par_loop(op2.Kernel(K2_MAX, "k"), s, g(op2.MAX), d2(op2.READ))
    assert g.data[0] == d2.data[:, 0].max() and g.data[1] == d2.data[:, 1].max()
    top = (d2.data[:, 0].max() + 1, d2.data[:, 1].max() + 1)
    g = op2.Global(2, top, dtype=np.uint32)
    op2.par_loop(op2.Kernel(K2_MAX, "k"), s, g(op2.MAX), d2(op2.READ))
    assert tuple(g.data) == top
    d2.data[:, 0] += 10
    d2.data[:, 1] += 10
    low = (d2.data[:, 0].min() - 1, d2.data[:, 1].min() - 1)
    g = op2.Global(2, low, dtype=np.uint32)
    op2.par_loop(op2.Kernel(K2_MIN, "k"), s, g(op2.MIN), d2(op2.READ))
    assert tuple(g.data) == low


def test_multi_inc(env):
    op2, s, dset, d1, d2 = env
    k = op2.Kernel(K1_INC, "k")
    g = op2.Global(1, 0, dtype=np.uint32)
    op2.par_loop(k, s, g(op2.INC), d1(op2.READ))
    assert g.data == d1.data.sum()
    op2.par_loop(k, s, g(op2.INC), d1(op2.READ))
    assert g.data == d1.data.sum() * 2
    g.data = 10
    op2.par_loop(k, s, g(op2.INC), d1(op2.READ))
    assert g.data == d1.data.sum() + 10
    g2 = op2.Global(1, 10, dtype=np.uint32)
    op2.par_loop(k, s, g2(op2.INC), d1(op2.READ))
    assert g2.data == d1.data.sum() + 10


def test_globals_with_different_types(env):
    op2, s, dset, d1, d2 = env
    g_uint32 = op2.Global(1, [0], np.uint32, "g_uint32")
    g_double = op2.Global(1, [0.0], np.float64, "g_double")
    op2.par_loop(op2.Kernel("static void k(unsigned int* i, double* d) { *i += 1; *d += 1.0f; }",
                            "k"), s, g_uint32(op2.INC), g_double(op2.INC))
    assert_allclose(g_uint32.data[0], g_double.data[0])
    assert g_uint32.data[0] == s.size


def test_inc_repeated_and_reused_loop(env):
    op2, s, dset, d1, d2 = env
    g = op2.Global(1, 0, dtype=np.uint32)
    k = "static void k(unsigned int* g) { *g += 1; }"
    op2.par_loop(op2.Kernel(k, "k"), s, g(op2.INC))
    assert_allclose(g.data, s.size)
    op2.par_loop(op2.Kernel(k, "k"), s, g(op2.INC))
    assert_allclose(g.data, 2 * s.size)
    g.zero()
    op2.par_loop(op2.Kernel(k, "k"), s, g(op2.INC))
    assert_allclose(g.data, s.size)
    g = op2.Global(1, 0, dtype=np.uint32)
    loop = op2.ParLoop(op2.Kernel("void k(unsigned int* g) { *g += 1; }", "k"), s, g(op2.INC))
    loop.compute()
    assert_allclose(g.data, s.size)
    loop.compute()
    assert_allclose(g.data, 2 * s.size)
    g.zero()
    loop.compute()
    assert_allclose(g.data, s.size)
