"""The non-legacy loop interface (pyop2/global_kernel.py, pyop2/parloop.py
:30-260): GlobalKernel + *KernelArg descriptors, Parloop over *ParloopArgs,
replace_data."""
import numpy as np
import pytest

from pyop2_gb300 import op2

gpu = pytest.mark.gpu


def _setup():
    cells, verts = op2.Set(6), op2.Set(8)
    vals = np.array([[0, 1, 2], [1, 2, 3], [2, 3, 4], [3, 4, 5], [4, 5, 6], [5, 6, 7]])
    m = op2.Map(cells, verts, 3, vals)
    x = op2.Dat(verts, np.arange(8.0))
    y = op2.Dat(verts, np.zeros(8))
    g = op2.Global(1, 0.0)
    return cells, verts, m, x, y, g, vals


def test_global_kernel_validation():
    cells, verts, m, x, y, g, vals = _setup()
    k = op2.Kernel("static void k(double *y, const double *x) {}", "k",
                   accesses=(op2.INC, op2.READ))
    gk = op2.GlobalKernel(k, (op2.DatKernelArg((1,), m._global_kernel_arg),
                              op2.DatKernelArg((1,), m._global_kernel_arg)))
    assert gk.name == "wrap_k"
    with pytest.raises(ValueError):       # argument count differs from the accesses
        op2.GlobalKernel(k, (op2.DatKernelArg((1,), None),))
    with pytest.raises(ValueError):
        op2.GlobalKernel(k, gk.arguments, pass_layer_arg=True)
    with pytest.raises(ValueError):       # argument count differs from the kernel's
        op2.Parloop(gk, cells, [op2.DatParloopArg(y, m)])


def test_legacy_loop_exposes_its_global_kernel():
    cells, verts, m, x, y, g, vals = _setup()
    k = op2.Kernel("static void k(double *y, const double *x) {}", "k")
    pl = op2.ParLoop(k, cells, y(op2.INC, m), x(op2.READ, m), g(op2.INC))
    gk = pl.global_kernel
    assert [type(a).__name__ for a in gk.arguments] == \
        ["DatKernelArg", "DatKernelArg", "GlobalKernelArg"]
    assert gk.arguments[0].map_.arity == 3
    assert isinstance(y(op2.INC, m).parloop_arg, op2.DatParloopArg)


def test_constants_are_read_only():
    cells, verts, m, x, y, g, vals = _setup()
    c = op2.Constant(1, 2.0)
    k = op2.Kernel("static void k(double *c) {}", "k", accesses=(op2.INC,))
    gk = op2.GlobalKernel(k, (op2.GlobalKernelArg((1,)),))
    with pytest.raises(ValueError):
        op2.Parloop(gk, cells, [op2.GlobalParloopArg(c)])


@gpu
def test_new_style_parloop_runs_and_replaces_data(gpu_op2):
    cells, verts, m, x, y, g, vals = _setup()
    k = op2.Kernel("""static void k(double *y, const double *x, double *s) {
        for (int i = 0; i < 3; ++i) { y[i] += x[i]; s[0] += x[i]; } }""", "k",
                   accesses=(op2.INC, op2.READ, op2.INC))
    gk = op2.GlobalKernel(k, (op2.DatKernelArg((1,), m._global_kernel_arg),
                              op2.DatKernelArg((1,), m._global_kernel_arg),
                              op2.GlobalKernelArg((1,))))
    pl = op2.Parloop(gk, cells, [op2.DatParloopArg(y, m), op2.DatParloopArg(x, m),
                                 op2.GlobalParloopArg(g)])
    pl.compute()
    expect = np.zeros(8)
    np.add.at(expect, vals.reshape(-1), np.arange(8.0)[vals.reshape(-1)])
    assert np.array_equal(y.data_ro, expect)
    assert g.data_ro[0] == np.arange(8.0)[vals].sum()
    assert pl.arguments[0].data is y
    # the same loop on another output Dat
    y2 = op2.Dat(verts, np.zeros(8))
    pl.replace_data(0, y2)
    pl.compute()
    assert np.array_equal(y2.data_ro, expect) and np.array_equal(y.data_ro, expect)
    assert pl.arguments[0].data is y2


def test_global_kernel_key_sees_shared_maps():
    """Two arguments through one map give another key than two arguments
    through two maps of the same shape (the map table entry is shared)."""
    cells, verts, m, x, y, g, vals = _setup()
    m2 = op2.Map(cells, verts, 3, vals)
    k = op2.Kernel("static void k(double *y, const double *x) {}", "k",
                   accesses=(op2.INC, op2.READ))
    same = op2.GlobalKernel(k, (op2.DatKernelArg((1,), m._global_kernel_arg),
                                op2.DatKernelArg((1,), m._global_kernel_arg)))
    same2 = op2.GlobalKernel(k, (op2.DatKernelArg((1,), m._global_kernel_arg),
                                 op2.DatKernelArg((1,), m._global_kernel_arg)))
    other = op2.GlobalKernel(k, (op2.DatKernelArg((1,), m._global_kernel_arg),
                                 op2.DatKernelArg((1,), m2._global_kernel_arg)))
    assert same.cache_key == same2.cache_key
    assert same.cache_key != other.cache_key
    assert op2.DatKernelArg((1,), m._global_kernel_arg) == \
        op2.DatKernelArg((1,), m._global_kernel_arg)
    with pytest.raises(ValueError):
        op2.MapKernelArg(3, offset=[1, 1, 1])          # unhashable offset
    with pytest.raises(TypeError):
        op2.ComposedMapKernelArg(object())
    with pytest.raises(AttributeError):
        m._global_kernel_arg.arity = 4                  # descriptors are immutable
