"""test/unit/test_direct_loop.py on the GPU: direct loops, Global reductions
through direct loops, host writes between loops, C++ kernels, passthrough
handles.

Consolidated tests and the reference tests they restate: test_global_max_min
-- test_global_{max,min}_dat_is_{max,min}, test_global_{max,min}_g_is_{max,min};
test_zero_dats -- test_zero_1d_dat, test_zero_2d_dat; test_passthrough_handle
-- test_passthrough_mat (a device array in place of the PETSc Mat)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NEL = 4096


@pytest.fixture(params=[(NEL, NEL, NEL), (0, NEL, NEL), (NEL // 2, NEL, NEL),
                        (0, NEL // 2, NEL)])
def env(request, gpu_op2):
    op2 = gpu_op2
    elems = op2.Set(request.param, "elems")
    xarray = np.arange(NEL, dtype=np.uint32)
    x = op2.Dat(op2.DataSet(elems, 1, "delems"), xarray, np.uint32, "x")
    y = op2.Dat(op2.DataSet(elems, 2, "delems2"), np.stack([xarray, xarray]).T.copy(), np.uint32,
                "x")
    g = op2.Global(1, 0, np.uint32, "g")
    h = op2.Global(1, 1, np.uint32, "h")
    return op2, elems, x, y, g, h


def test_wo(env):
    op2, elems, x, y, g, h = env
    op2.par_loop(op2.Kernel("static void wo(unsigned int* x) { *x = 42; }", "wo"), elems,
                 x(op2.WRITE))
    assert all(v == 42 for v in x.data)


def test_mismatch_set_raises_error(env):
    op2, elems, x, y, g, h = env
    from pyop2_gb300.exceptions import MapValueError
    with pytest.raises(MapValueError):
        op2.par_loop(op2.Kernel("static void wo(unsigned int* x) { *x = 42; }", "wo"),
                     op2.Set(elems.size), x(op2.WRITE))


def test_rw(env):
    op2, elems, x, y, g, h = env
    op2.par_loop(op2.Kernel("static void wo(unsigned int* x) { (*x) = (*x) + 1; }", "wo"),
                 elems, x(op2.RW))
    n = elems.size
    assert sum(x.data_ro) == n * (n + 1) // 2
    if n == NEL:
        assert sum(x.data_ro_with_halos) == NEL * (NEL + 1) // 2


def test_global_inc(env):
    op2, elems, x, y, g, h = env
    k = """static void global_inc(unsigned int* x, unsigned int* inc) {
      (*x) = (*x) + 1; (*inc) += (*x); }"""
    op2.par_loop(op2.Kernel(k, "global_inc"), elems, x(op2.RW), g(op2.INC))
    n = elems.size
    assert g.data[0] == n * (n + 1) // 2


def test_global_inc_init_not_zero(env):
    op2, elems, x, y, g, h = env
    g.data[0] = 10
    op2.par_loop(op2.Kernel("static void k(unsigned int* inc) { (*inc) += 1; }", "k"), elems,
                 g(op2.INC))
    assert g.data[0] == elems.size + 10


def test_global_max_min(env):
    op2, elems, x, y, g, h = env
    kmax_g_first = "static void k(unsigned int *g, unsigned int *x) { if (*g < *x) { *g = *x; } }"
    op2.par_loop(op2.Kernel(kmax_g_first, "k"), elems, g(op2.MAX), x(op2.READ))
    assert g.data[0] == x.data.max()
    kmax = "static void k(unsigned int *x, unsigned int *g) { if (*g < *x) { *g = *x; } }"
    g.data[0] = NEL * 2
    op2.par_loop(op2.Kernel(kmax, "k"), elems, x(op2.READ), g(op2.MAX))
    assert g.data[0] == NEL * 2
    kmin_g_first = "static void k(unsigned int *g, unsigned int *x) { if (*g > *x) { *g = *x; } }"
    g.data[0] = 1000
    op2.par_loop(op2.Kernel(kmin_g_first, "k"), elems, g(op2.MIN), x(op2.READ))
    assert g.data[0] == x.data.min()
    kmin = "static void k(unsigned int *x, unsigned int *g) { if (*g > *x) { *g = *x; } }"
    g.data[0] = 10
    x.data[:] = 11
    op2.par_loop(op2.Kernel(kmin, "k"), elems, x(op2.READ), g(op2.MIN))
    assert g.data[0] == 10


def test_global_read(env):
    op2, elems, x, y, g, h = env
    op2.par_loop(op2.Kernel("static void global_read(unsigned int* x, unsigned int* h) "
                            "{ (*x) += (*h); }", "global_read"), elems, x(op2.RW), h(op2.READ))
    n = elems.size
    assert sum(x.data_ro) == n * (n + 1) // 2


def test_2d_dat(env):
    op2, elems, x, y, g, h = env
    op2.par_loop(op2.Kernel("static void k2d_wo(unsigned int* x) { x[0] = 42; x[1] = 43; }",
                            "k2d_wo"), elems, y(op2.WRITE))
    assert all(all(v == [42, 43]) for v in y.data)


def test_host_write(env):
    op2, elems, x, y, g, h = env
    x.data[:] = 1
    g.data[:] = 0
    op2.par_loop(op2.Kernel("static void k(unsigned int *g, unsigned int *x) { *g += *x; }", "k"),
                 elems, g(op2.INC), x(op2.READ))
    assert g.data[0] == elems.size
    x.data[:] = 2
    g.data[:] = 0
    op2.par_loop(op2.Kernel("static void k(unsigned int *x, unsigned int *g) { *g += *x; }", "k"),
                 elems, x(op2.READ), g(op2.INC))
    assert g.data[0] == 2 * elems.size


def test_zero_dats(env):
    op2, elems, x, y, g, h = env
    for d in (x, y):
        d.data[:] = 10
        assert (d.data == 10).all()
        d.zero()
        assert (d.data == 0).all()


def test_kernel_cplusplus(gpu_op2):
    op2 = gpu_op2
    y = op2.Dat(op2.DataSet(op2.Set(NEL), 1), dtype=np.float64)
    y.data[:] = -10.5
    k = op2.Kernel("""
    #include <cmath>

    static void k(double *y)
    {
        *y = std::abs(*y);
    }
    """, "k", cpp=True)
    op2.par_loop(k, y.dataset.set, y(op2.RW))
    assert (y.data == 10.5).all()


def test_passthrough_handle(gpu_op2):
    """A raw handle reaches the kernel untouched (the reference passes a PETSc
    Mat this way); here it is a device array the kernel adds into."""
    import torch
    op2 = gpu_op2
    from pyop2_gb300 import device
    buf = torch.zeros(9, dtype=torch.float64, device=device.device())
    kernel = op2.Kernel("""
    typedef double *Handle;
    static void add_block(Handle h) {
      const double v[] = {1, 2, 3, 4, 5, 6, 7, 8, 9};
      for (int i = 0; i < 9; ++i) atomicAdd(&h[i], v[i]);
    }""", "add_block")
    op2.par_loop(kernel, op2.Set(10), op2.PassthroughArg(op2.OpaqueType("Handle"),
                                                         buf.data_ptr()))
    assert np.allclose(buf.cpu().numpy(), 10 * np.arange(1, 10))
