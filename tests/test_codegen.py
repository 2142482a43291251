"""Wrapper generation and NVRTC compilation for sm_103a, on CPU (NVRTC needs
no GPU when the architecture is given).  Covers every access mode, element
type, Global reductions, Mats, extruded regions, permuted and composed maps
and the three INC strategies."""
import numpy as np
import pytest

from pyop2_gb300 import _lib
from pyop2_gb300.parloop import LegacyParloop, compile_signature


@pytest.fixture(scope="module")
def op2():
    from pyop2_gb300.csrc import build
    build.build()
    from pyop2_gb300 import op2
    return op2


def compile_loop(pl, scatter=_lib.SCATTER_ATOMIC, bs=256):
    table, argdescs = pl._signature()
    loop = pl._loop_desc(scatter, bs)
    return compile_signature(pl.local_kernel.source, pl.local_kernel.name, loop, argdescs,
                             table.key(), arch="sm_103a")


@pytest.mark.parametrize("scatter", [_lib.SCATTER_ATOMIC, _lib.SCATTER_WARP, _lib.SCATTER_PLAIN,
                                     _lib.SCATTER_STAGED])
@pytest.mark.parametrize("dtype,ctype", [(np.float64, "double"), (np.float32, "float"),
                                         (np.int32, "int"), (np.uint32, "unsigned int"),
                                         (np.int64, "long long")])
def test_all_access_modes(op2, scatter, dtype, ctype):
    cells, verts = op2.Set(8), op2.Set(10)
    m = op2.Map(cells, verts, 3, np.arange(24) % 10)
    dats = [op2.Dat(verts ** 2, dtype=dtype) for _ in range(6)]
    direct = op2.Dat(cells, dtype=dtype)
    g = [op2.Global(2, dtype=dtype) for _ in range(4)]
    src = "static void k(%s) {}" % ", ".join(["%s *a%d" % (ctype, i) for i in range(11)])
    k = op2.Kernel(src, "k")
    pl = LegacyParloop(k, cells, dats[0](op2.READ, m), dats[1](op2.WRITE, m), dats[2](op2.RW, m),
                       dats[3](op2.INC, m), dats[4](op2.MIN, m), dats[5](op2.MAX, m),
                       direct(op2.RW), g[0](op2.READ), g[1](op2.INC), g[2](op2.MIN), g[3](op2.MAX))
    c = compile_loop(pl, scatter)
    assert c.nptrs == 12
    s = c.source()
    assert "op2g_wrap" in s and "op2g_wrap_batched" in s
    if scatter == _lib.SCATTER_WARP:
        assert "warp_agg_inc" in s
    if scatter == _lib.SCATTER_STAGED:
        # READ (no written Dat is read) and INC are staged, nothing else
        assert "op2g_run_staged" in s and "sv0[" in s and "sv3[" in s
        assert not any("sv%d[" % a in s for a in (1, 2, 4, 5, 6))
        assert "op2g_wrap_chunked" not in s


def test_staged_wrapper_stages_reads_and_incs(op2):
    """A staged gather/scatter loop through a plain and a permuted map: READ
    and INC values come from and go to shared memory at local indices."""
    cells, verts = op2.Set(8), op2.Set(10)
    m = op2.Map(cells, verts, 4, np.arange(32) % 10)
    pm = op2.PermutedMap(m, [1, 0, 3, 2])
    x = op2.Dat(verts ** 3, dtype=np.float64)
    y = op2.Dat(verts, dtype=np.float64)
    z = op2.Dat(verts, dtype=np.float32)
    w = op2.Dat(cells, dtype=np.float64)
    k = op2.Kernel("static void k(double *y, const double *x, float *z, const double *w) {}", "k")
    pl = LegacyParloop(k, cells, y(op2.INC, m), x(op2.READ, pm), z(op2.INC, pm), w(op2.READ))
    s = compile_loop(pl, _lib.SCATTER_STAGED).source()
    assert "op2g_run_staged" in s
    for a in (0, 1, 2):
        assert "sv%d[" % a in s
    assert "op2g_perm1" in s and "lv0[" in s and "ushort4" in s


@pytest.mark.parametrize("region", [1, 2, 3, 4])
@pytest.mark.parametrize("constant", [True, False])
@pytest.mark.parametrize("periodic", [False, True])
def test_extruded_regions(op2, region, constant, periodic):
    base = op2.Set(4)
    layers = 5 if constant else np.array([[0, 5], [1, 4], [0, 3], [2, 5]])
    ext = op2.ExtrudedSet(base, layers, extruded_periodic=periodic)
    nodes = op2.Set(5 * 6)
    m = op2.Map(ext, nodes, 2, np.arange(8) % 6 * 5, offset=[1, 1],
                offset_quotient=[0, 1] if periodic else None)
    d = op2.Dat(nodes, dtype=np.float64)
    k = op2.Kernel("static void k(double *y, int layer) { y[0] += layer; }", "k")
    pl = LegacyParloop(k, ext, d(op2.INC, m), iteration_region=region, pass_layer_arg=True)
    c = compile_loop(pl)
    assert "layer" in c.source()


def test_mat_argument(op2):
    cells, verts = op2.Set(2), op2.Set(4)
    m = op2.Map(cells, verts, 3, [0, 1, 3, 2, 3, 1])
    from pyop2_gb300.parloop import MatLegacyArg

    class FakeMat:  # signature only: no device needed to generate code
        dtype = np.dtype(np.float64)
        dims = (((2, 2),),)
    k = op2.Kernel("static void k(double A[6][6]) {}", "k")
    for acc in (op2.INC, op2.WRITE):
        pl = LegacyParloop(k, cells, MatLegacyArg(FakeMat(), (m, m), acc))
        src = compile_loop(pl).source()
        assert "bcsr_find" in src


def test_permuted_and_composed_maps(op2):
    setB, nodesetB = op2.Set(3), op2.Set(6)
    setA, nodesetA = op2.Set(5), op2.Set(8)
    mapB = op2.Map(setB, nodesetB, 2, [[0, 1], [2, 3], [4, 5]])
    mapA0 = op2.Map(setA, nodesetA, 2, [[0, 1], [2, 3], [4, 5], [6, 7], [0, 1]])
    mapA1 = op2.Map(setB, setA, 1, [3, 1, 2])
    cm = op2.ComposedMap(op2.PermutedMap(mapA0, [1, 0]), mapA1)
    dB = op2.Dat(nodesetB)
    dA = op2.Dat(nodesetA)
    k = op2.Kernel("void copy(double *to, const double * restrict from) { to[0] = from[0]; }",
                   "copy")
    pl = LegacyParloop(k, setB, dB(op2.WRITE, op2.PermutedMap(mapB, [1, 0])), dA(op2.READ, cm))
    src = compile_loop(pl).source()
    assert "op2g_perm" in src


def test_compile_error_is_a_compilation_error(op2):
    from pyop2_gb300.exceptions import CompilationError
    s = op2.Set(4)
    d = op2.Dat(s)
    pl = LegacyParloop(op2.Kernel("static void k(double *x) { this is not C; }", "k"), s,
                       d(op2.WRITE))
    with pytest.raises(CompilationError) as e:
        compile_loop(pl)
    assert "generated source" in str(e.value)


def test_mixed_arguments_share_one_parameter(op2):
    """MixedDat and mixed-Mat components form one kernel parameter
    (pyop2/codegen/builder.py:413-498, 609-680)."""
    from pyop2_gb300.parloop import MixedMatLegacyArg
    elem, node = op2.Set(3), op2.Set(4)
    mmap = op2.MixedMap((op2.Map(elem, elem, 1, [0, 1, 2]),
                         op2.Map(elem, node, 2, [0, 1, 1, 2, 2, 3])))
    mdat = op2.MixedDat([op2.Dat(elem), op2.Dat(node)])

    class Block:
        dtype = np.dtype(np.float64)

        def __init__(self, rd, cd):
            self.dims = (((rd, cd),),)

    class FakeMixedMat:
        dtype = np.dtype(np.float64)

        class sparsity:
            shape = (2, 2)

        def __getitem__(self, ij):
            return Block(1, 1)
    k = op2.Kernel("static void addone_mat(double v[9], double d[3]) {}", "addone_mat")
    pl = LegacyParloop(k, elem, MixedMatLegacyArg(FakeMixedMat(), (mmap, mmap), op2.INC),
                       mdat(op2.READ, mmap))
    src = compile_loop(pl).source()
    # one 3 x 3 element matrix and one 3-entry pack reach the kernel
    assert "double t0[9];" in src and "double t4[3];" in src
    assert "addone_mat(op2g::ptr(t0), op2g::ptr(t4));" in src
    # block (1, 1) reads rows 1.. and columns 1.. of the 3-wide element matrix
    assert "t0[(1 + (0 + i) * 1 + ri) * 3 + 1 + (0 + j) * 1 + cj]" in src


def _raw_compile(args, maps=((_lib.MAP_PLAIN, 2, -1, (), None, None, None),)):
    loop = dict(extruded=0, constant_layers=0, extruded_periodic=0, indexed=0,
                iteration_region=4, pass_layer_arg=0, scatter=0, block_size=256,
                debug_checks=0, batched=0)
    return compile_signature("static void k(double *a) {}", "k", loop, args, list(maps),
                             arch="sm_103a")


@pytest.mark.parametrize("args,msg", [
    # a group split by another argument
    ([(0, 4, 0, 1, 0, -1, 0, 0, 1, 0), (0, 1, 0, 1, -1, -1, 0, 0, 0, 0),
      (0, 4, 0, 1, 0, -1, 0, 0, 1, 0)], "not contiguous"),
    # components of one group with different access
    ([(0, 4, 0, 1, 0, -1, 0, 0, 1, 0), (0, 1, 0, 1, 0, -1, 0, 0, 1, 0)], "one kind"),
    # a direct component
    ([(0, 4, 0, 1, 0, -1, 0, 0, 1, 0), (0, 4, 0, 1, -1, -1, 0, 0, 1, 0)], "indirect"),
    # three Mat blocks cannot form two block columns
    ([(2, 4, 0, 1, 0, 0, 1, 1, 1, 2)] * 3, "group_cols"),
    # a grouped Global
    ([(1, 4, 0, 1, -1, -1, 0, 0, 1, 0)] * 2, "only Dats and Mats"),
])
def test_bad_groups_are_rejected(op2, args, msg):
    with pytest.raises(_lib.Op2gError) as e:
        _raw_compile(args)
    assert msg in str(e.value)


@pytest.mark.parametrize("decl", ["static void k()", "static void k( void )", "void k ( )"])
def test_kernel_with_empty_parameter_list(op2, decl):
    """C leaves the parameters of `k()` unspecified, so the reference may
    pass arguments to it (test/unit/test_api.py:278-286); the wrapper then
    calls it without arguments."""
    cells, verts = op2.Set(4), op2.Set(5)
    m = op2.Map(cells, verts, 2, np.arange(8) % 5)
    d = op2.Dat(verts)
    pl = LegacyParloop(op2.Kernel(decl + " { }", "k"), cells, d(op2.READ, m))
    assert "k();" in compile_loop(pl).source()
    pl2 = LegacyParloop(op2.Kernel("static void kk(double *x) { }", "kk"), cells, d(op2.READ, m))
    assert "kk(op2g::ptr(t0));" in compile_loop(pl2).source()


@pytest.mark.parametrize("cells", [1, 2, 3])
def test_cells_per_thread(op2, cells):
    """Several cells per thread: the unpack (INC, Globals) is guarded,
    the gathers and the call are not; loops that update a direct argument
    (RW, INC) fall back to one cell per thread, direct WRITE arguments do not
    (the rerun last iteration stores the same values)."""
    cells_, verts = op2.Set(8), op2.Set(10)
    m = op2.Map(cells_, verts, 3, np.arange(24) % 10)
    x, y = op2.Dat(verts ** 2), op2.Dat(verts)
    g = op2.Global(1, 0.0)
    k = op2.Kernel("static void k(double *y, const double *x, double *g) {}", "k")
    pl = LegacyParloop(k, cells_, y(op2.INC, m), x(op2.READ, m), g(op2.MIN))
    table, argdescs = pl._signature()
    src = compile_signature(pl.local_kernel.source, "k", pl._loop_desc(_lib.SCATTER_ATOMIC, 256, 0, cells),
                            argdescs, table.key(), arch="sm_103a").source()
    if cells > 1:
        assert "stride * %d" % cells in src and "i1_ - 1" in src and "if (active) {" in src
    else:
        assert "stride * " not in src
    d = op2.Dat(cells_)
    for acc, multi in ((op2.WRITE, cells > 1), (op2.RW, False), (op2.INC, False)):
        pl2 = LegacyParloop(op2.Kernel("static void k2(double *y, double *d) {}", "k2"), cells_,
                            y(op2.INC, m), d(acc))
        table, argdescs = pl2._signature()
        src2 = compile_signature(pl2.local_kernel.source, "k2",
                                 pl2._loop_desc(_lib.SCATTER_ATOMIC, 256, 0, cells),
                                 argdescs, table.key(), arch="sm_103a").source()
        assert ("stride * " in src2) == multi


def test_next_rows_of_read_direct_arguments_are_prefetched(op2):
    """A flat loop prefetches the next sweep step's rows of the direct
    arguments it reads (READ, RW) into L2, not of those it only writes; an
    indexed loop (a Subset: the next entity is not known) prefetches none."""
    cells = op2.Set(8)
    r, w, b = op2.Dat(cells ** 2), op2.Dat(cells ** 3), op2.Dat(cells)
    k = op2.Kernel("static void k(const double *r, double *w, double *b) {}", "k")
    src = compile_loop(LegacyParloop(k, cells, r(op2.READ), w(op2.WRITE), b(op2.RW))).source()
    assert src.count("prefetch.global.L2") == 2
    assert "(double *)p.ptr[0] + (it + stride) * 2" in src
    assert "(double *)p.ptr[2] + (it + stride) * 1" in src
    assert "p.ptr[1] + (it + stride)" not in src
    sub = op2.Subset(cells, [1, 3, 5])
    src2 = compile_loop(LegacyParloop(k, sub, r(op2.READ), w(op2.WRITE), b(op2.RW))).source()
    assert "prefetch.global.L2" not in src2


def test_inc_packs_start_at_negative_zero(op2):
    """INC packs of floating types (Dat, Mat, Global) start at -0.0, the
    identity of IEEE addition; WRITE packs and integer INC packs at 0."""
    cells, verts = op2.Set(8), op2.Set(10)
    m = op2.Map(cells, verts, 2, np.arange(16) % 10)
    yd, yf, yi, wd = (op2.Dat(verts, dtype=np.float64), op2.Dat(verts, dtype=np.float32),
                      op2.Dat(verts, dtype=np.int32), op2.Dat(verts, dtype=np.float64))
    g = op2.Global(1, 0.0)
    k = op2.Kernel("static void k(double *a, float *b, int *c, double *d, double *g) {}", "k")
    src = compile_loop(LegacyParloop(k, cells, yd(op2.INC, m), yf(op2.INC, m), yi(op2.INC, m),
                                     wd(op2.WRITE, m), g(op2.INC))).source()
    assert "t0[k] = (-0.0);" in src and "t1[k] = (-0.0f);" in src
    assert "t2[k] = (int)0;" in src and "t3[k] = (double)0;" in src
    assert "g4[j] = (-0.0);" in src
