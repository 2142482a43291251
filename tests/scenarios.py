"""Problem scenarios shared by the oracle tests (CPU) and the GPU parity tests.

Each ``sc_*`` function takes an ``op2`` module -- pyop2_gb300.op2 or the
oracle -- builds a small problem the way the reference's unit tests do, runs
it, and asserts the values those tests assert (their expected results are
the golden vectors; the reference test each one follows is cited).  Some
scenarios return arrays so a test can also compare implementations
directly.

Reference tests by name (test/unit/...) and the scenario restating each:

    test_indirect_loop.py  test_onecolor_wo -> sc_indirect_wo,
        test_onecolor_rw -> sc_indirect_rw, test_indirect_inc / _max / _min
        -> sc_indirect_inc / _max / _min, test_global_read / _inc ->
        sc_global_read / _inc, test_2d_dat -> sc_2d_dat, test_2d_map ->
        sc_2d_map, test_mixed_non_mixed_dat(_itspace) ->
        sc_mixed_non_mixed_dat, test_permuted_map / _both -> sc_permuted_map /
        sc_permuted_map_both, test_composed_map_two_maps /
        _three_maps -> sc_composed_two_maps / sc_composed_three_maps
    test_iteration_space_dats.py  test_sum_nodes_to_edges ->
        sc_itspace_sum_nodes_to_edges; test_{read,write,inc}_{1d,2d}_itspace_map
        -> sc_vm_{read,write,inc}_{1d,2d} (the same loops through arity-1 maps)
    test_vector_map.py  test_{read,write,inc}_{1d,2d}_vector_map ->
        sc_vm_{read,write,inc}_{1d,2d}
    test_extrusion.py  test_direct_loop_inc -> sc_extrusion_direct_inc,
        test_extruded_layer_arg -> sc_extrusion_layer_arg,
        test_indirect_coords_inc -> sc_extrusion_write_coords, the volume and
        field tests -> sc_extrusion_volume, sc_extrusion_fields
"""
import numpy as np
from numpy.testing import assert_allclose

NELEMS = 4096

SIZES = [(NELEMS, NELEMS, NELEMS), (0, NELEMS, NELEMS), (NELEMS // 2, NELEMS, NELEMS)]


# ------------------------------------------------------------------------
# test/unit/test_indirect_loop.py:46-232
def _indirect_fixtures(op2, sizes):
    iterset = op2.Set(sizes, "iterset")
    indset = op2.Set(NELEMS, "indset")
    x = op2.Dat(indset, np.arange(NELEMS), np.uint32, "x")
    mapd = np.arange(NELEMS)[::-1]
    m = op2.Map(iterset, indset, 1, mapd.astype(np.uint32), "iterset2indset")
    return iterset, indset, x, m


def sc_indirect_wo(op2, sizes=SIZES[0]):
    iterset, indset, x, m = _indirect_fixtures(op2, sizes)
    op2.par_loop(op2.Kernel("static void kernel_wo(unsigned int* x) { *x = 42; }\n", "kernel_wo"),
                 iterset, x(op2.WRITE, m))
    assert np.all(x.data == 42)


def sc_indirect_rw(op2, sizes=SIZES[0]):
    iterset, indset, x, m = _indirect_fixtures(op2, sizes)
    op2.par_loop(op2.Kernel("static void rw(unsigned int* x) { (*x) = (*x) + 1; }\n", "rw"),
                 iterset, x(op2.RW, m))
    assert int(np.sum(x.data, dtype=np.int64)) == NELEMS * (NELEMS + 1) // 2


def sc_indirect_inc(op2, sizes=SIZES[0]):
    iterset = op2.Set(sizes, "iterset")
    unitset = op2.Set(1, "unitset")
    u = op2.Dat(unitset, np.array([0], dtype=np.uint32), np.uint32, "u")
    m = op2.Map(iterset, unitset, 1, np.zeros(NELEMS, dtype=np.uint32), "iterset2unitset")
    op2.par_loop(op2.Kernel("static void inc(unsigned int* x) { (*x) = (*x) + 1; }\n", "inc"),
                 iterset, u(op2.INC, m))
    assert u.data[0] == NELEMS


def sc_indirect_max(op2, sizes=SIZES[0]):
    iterset, indset, x, m = _indirect_fixtures(op2, sizes)
    a = op2.Dat(indset, dtype=np.int32)
    b = op2.Dat(indset, dtype=np.int32)
    a.data[:] = -10
    b.data[:] = -5
    k = "static void maxify(int *a, int *b) {*a = *a < *b ? *b : *a;}\n"
    op2.par_loop(op2.Kernel(k, "maxify"), iterset, a(op2.MAX, m), b(op2.READ, m))
    assert np.all(a.data_ro == -5)


def sc_indirect_min(op2, sizes=SIZES[0]):
    iterset, indset, x, m = _indirect_fixtures(op2, sizes)
    a = op2.Dat(indset, dtype=np.int32)
    b = op2.Dat(indset, dtype=np.int32)
    a.data[:] = 10
    b.data[:] = 5
    k = "static void minify(int *a, int *b) {*a = *a > *b ? *b : *a;}\n"
    op2.par_loop(op2.Kernel(k, "minify"), iterset, a(op2.MIN, m), b(op2.READ, m))
    assert np.all(a.data_ro == 5)


def sc_global_read(op2, sizes=SIZES[0]):
    iterset, indset, x, m = _indirect_fixtures(op2, sizes)
    g = op2.Global(1, 2, np.uint32, "g")
    k = "static void global_read(unsigned int* x, unsigned int* g) { (*x) /= (*g); }\n"
    op2.par_loop(op2.Kernel(k, "global_read"), iterset, x(op2.RW, m), g(op2.READ))
    assert int(np.sum(x.data, dtype=np.int64)) == sum(v // 2 for v in range(NELEMS))


def sc_global_inc(op2, sizes=SIZES[0]):
    iterset, indset, x, m = _indirect_fixtures(op2, sizes)
    g = op2.Global(1, 0, np.uint32, "g")
    k = """
    static void global_inc(unsigned int *x, unsigned int *inc) {
      (*x) = (*x) + 1; (*inc) += (*x);
    }"""
    op2.par_loop(op2.Kernel(k, "global_inc"), iterset, x(op2.RW, m), g(op2.INC))
    assert int(np.sum(x.data, dtype=np.int64)) == NELEMS * (NELEMS + 1) // 2
    assert g.data[0] == NELEMS * (NELEMS + 1) // 2


def sc_2d_dat(op2, sizes=SIZES[0]):
    iterset, indset, x, m = _indirect_fixtures(op2, sizes)
    x2 = op2.Dat(op2.DataSet(indset, 2), np.array([np.arange(NELEMS), np.arange(NELEMS)],
                                                   dtype=np.uint32).T.copy(), np.uint32, "x2")
    k = "static void wo(unsigned int* x) { x[0] = 42; x[1] = 43; }\n"
    op2.par_loop(op2.Kernel(k, "wo"), iterset, x2(op2.WRITE, m))
    assert np.all(x2.data[:, 0] == 42) and np.all(x2.data[:, 1] == 43)


def sc_2d_map(op2):
    nedges = NELEMS - 1
    nodes = op2.Set(NELEMS, "nodes")
    edges = op2.Set(nedges, "edges")
    node_vals = op2.Dat(nodes, np.arange(NELEMS, dtype=np.uint32), np.uint32, "node_vals")
    edge_vals = op2.Dat(edges, np.zeros(nedges, dtype=np.uint32), np.uint32, "edge_vals")
    e_map = np.array([(i, i + 1) for i in range(nedges)], dtype=np.uint32)
    edge2node = op2.Map(edges, nodes, 2, e_map, "edge2node")
    k = """
    static void sum(unsigned int *edge, unsigned int *nodes) {
      *edge = nodes[0] + nodes[1];
    }"""
    op2.par_loop(op2.Kernel(k, "sum"), edges, edge_vals(op2.WRITE), node_vals(op2.READ, edge2node))
    assert np.all(np.arange(1, nedges * 2 + 1, 2) == edge_vals.data)


# test/unit/test_iteration_space_dats.py:89-112 (INC into a direct Dat)
def sc_itspace_sum_nodes_to_edges(op2):
    nedges = NELEMS - 1
    nodes = op2.Set(NELEMS, "nodes")
    edges = op2.Set(nedges, "edges")
    node_vals = op2.Dat(nodes, np.arange(NELEMS, dtype=np.uint32), np.uint32, "node_vals")
    edge_vals = op2.Dat(edges, np.zeros(nedges, dtype=np.uint32), np.uint32, "edge_vals")
    e_map = np.array([(i, i + 1) for i in range(nedges)], dtype=np.uint32)
    edge2node = op2.Map(edges, nodes, 2, e_map, "edge2node")
    k = """
static void sum(unsigned int *edge, unsigned int *nodes) {
  for (int i=0; i<2; ++i)
    edge[0] += nodes[i];
}"""
    op2.par_loop(op2.Kernel(k, "sum"), edges, edge_vals(op2.INC), node_vals(op2.READ, edge2node))
    assert np.all(np.arange(1, nedges * 2 + 1, 2) == edge_vals.data)


# ------------------------------------------------------------------------
# test/unit/test_vector_map.py:45-236 (node -> element map with arity 1)
def _vm(op2):
    nnodes = 4096
    nele = nnodes // 2
    node = op2.Set(nnodes, "node")
    ele = op2.Set(nele, "ele")
    d1 = op2.Dat(op2.DataSet(node, 1), np.zeros(nnodes), dtype=np.int32)
    d2 = op2.Dat(op2.DataSet(node, 2), np.zeros(2 * nnodes), dtype=np.int32)
    vd1 = op2.Dat(op2.DataSet(ele, 1), np.zeros(nele), dtype=np.int32)
    vd2 = op2.Dat(op2.DataSet(ele, 2), np.zeros(2 * nele), dtype=np.int32)
    node2ele = op2.Map(node, ele, 1, (np.arange(nnodes) // 2).astype(np.int32), "node2ele")
    return nnodes, nele, node, d1, d2, vd1, vd2, node2ele


def sc_vm_read_1d(op2):
    nnodes, nele, node, d1, d2, vd1, vd2, n2e = _vm(op2)
    vd1.data[:] = np.arange(nele)
    k = "static void k(int *d, int *vd) { *d = vd[0]; }"
    op2.par_loop(op2.Kernel(k, "k"), node, d1(op2.WRITE), vd1(op2.READ, n2e))
    assert np.all(d1.data[::2] == vd1.data) and np.all(d1.data[1::2] == vd1.data)


def sc_vm_write_1d(op2):
    nnodes, nele, node, d1, d2, vd1, vd2, n2e = _vm(op2)
    op2.par_loop(op2.Kernel("static void k(int *vd) { vd[0] = 2; }", "k"), node, vd1(op2.WRITE, n2e))
    assert np.all(vd1.data == 2)


def sc_vm_inc_1d(op2):
    nnodes, nele, node, d1, d2, vd1, vd2, n2e = _vm(op2)
    vd1.data[:] = 3
    d1.data[:] = np.arange(nnodes).reshape(d1.data.shape)
    k = "static void k(int *vd, int *d) { vd[0] += *d; }"
    op2.par_loop(op2.Kernel(k, "k"), node, vd1(op2.INC, n2e), d1(op2.READ))
    expected = 3 + np.arange(0, nnodes, 2) + np.arange(1, nnodes, 2)
    assert np.all(vd1.data == expected)


def sc_vm_read_2d(op2):
    nnodes, nele, node, d1, d2, vd1, vd2, n2e = _vm(op2)
    vd2.data[:] = np.arange(nele * 2).reshape(nele, 2)
    k = """static void k(int d[2], int vd[1][2]) { d[0] = vd[0][0]; d[1] = vd[0][1]; }"""
    op2.par_loop(op2.Kernel(k, "k"), node, d2(op2.WRITE), vd2(op2.READ, n2e))
    assert np.all(d2.data[::2] == vd2.data) and np.all(d2.data[1::2] == vd2.data)


def sc_vm_write_2d(op2):
    nnodes, nele, node, d1, d2, vd1, vd2, n2e = _vm(op2)
    k = "static void k(int vd[1][2]) { vd[0][0] = 2; vd[0][1] = 3; }"
    op2.par_loop(op2.Kernel(k, "k"), node, vd2(op2.WRITE, n2e))
    assert np.all(vd2.data[:, 0] == 2) and np.all(vd2.data[:, 1] == 3)


def sc_vm_inc_2d(op2):
    nnodes, nele, node, d1, d2, vd1, vd2, n2e = _vm(op2)
    vd2.data[:, 0] = 3
    vd2.data[:, 1] = 4
    d2.data[:] = np.arange(2 * nnodes).reshape(d2.data.shape)
    k = "static void k(int vd[1][2], int d[2]) { vd[0][0] += d[0]; vd[0][1] += d[1]; }"
    op2.par_loop(op2.Kernel(k, "k"), node, vd2(op2.INC, n2e), d2(op2.READ))
    e0 = 3 + np.arange(0, 2 * nnodes, 4) + np.arange(2, 2 * nnodes, 4)
    e1 = 4 + np.arange(1, 2 * nnodes, 4) + np.arange(3, 2 * nnodes, 4)
    assert np.all(vd2.data[:, 0] == e0) and np.all(vd2.data[:, 1] == e1)


# ------------------------------------------------------------------------
# test/unit/test_global_reduction.py:45-462
def _gr(op2, sizes):
    s = op2.Set(sizes, "set")
    d1 = op2.Dat(op2.DataSet(s, 1), np.arange(NELEMS) + 1, dtype=np.uint32)
    d2 = op2.Dat(op2.DataSet(s, 2), np.arange(2 * NELEMS) + 1, dtype=np.uint32)
    return s, d1, d2


K_INC = "static void k(unsigned int *g, unsigned int *x) { *g += *x; }"
K_MIN = "static void k(unsigned int *g, unsigned int *x) { if (*x < *g) *g = *x; }"
K_MAX = "static void k(unsigned int *g, unsigned int *x) { if (*x > *g) *g = *x; }"
K2_INC = "static void k(unsigned int *g, unsigned int *x) { g[0] += x[0]; g[1] += x[1]; }"
K2_MIN = """static void k(unsigned int *g, unsigned int *x) {
 if (x[0] < g[0]) g[0] = x[0]; if (x[1] < g[1]) g[1] = x[1]; }"""
K2_MAX = """static void k(unsigned int *g, unsigned int *x) {
 if (x[0] > g[0]) g[0] = x[0]; if (x[1] > g[1]) g[1] = x[1]; }"""


def sc_gr_direct_typed(op2, sizes=SIZES[0]):
    s = op2.Set(sizes, "set")
    cases = [(np.uint32, "unsigned int", 12, 8, op2.MIN, "<", 8),
             (np.int32, "int", -12, 8, op2.MIN, "<", -12),
             (np.int32, "int", -12, -42, op2.MAX, ">", -12),
             (np.float32, "float", -12.0, -.8, op2.MIN, "<", -12.0),
             (np.float32, "float", -12.0, -42.8, op2.MAX, ">", -12.0),
             (np.float64, "double", -12.0, -.8, op2.MIN, "<", -12.0),
             (np.float64, "double", -12.0, -42.8, op2.MAX, ">", -12.0)]
    for dt, ct, dval, gval, acc, cmp, expect in cases:
        d = op2.Dat(op2.DataSet(s, 1), [dval] * NELEMS, dt, "d")
        k = "static void k(%s* g, %s* x) { if ( *x %s *g ) *g = *x; }" % (ct, ct, cmp)
        g = op2.Global(1, gval, dt, "g")
        op2.par_loop(op2.Kernel(k, "k"), s, g(acc), d(op2.READ))
        assert_allclose(g.data[0], expect)


def sc_gr_read_and_inc(op2, sizes=SIZES[0]):
    s, d1, d2 = _gr(op2, sizes)
    g = op2.Global(1, 1, dtype=np.uint32)
    op2.par_loop(op2.Kernel("static void k(unsigned int *x, unsigned int *g) { *x = *g; }", "k"),
                 s, d1(op2.WRITE), g(op2.READ))
    assert np.all(d1.data == 1)
    g2 = op2.Global(2, (1, 2), dtype=np.uint32)
    op2.par_loop(op2.Kernel("static void k(unsigned int *x, unsigned int *g) { *x = g[0] + g[1]; }",
                            "k"), s, d1(op2.WRITE), g2(op2.READ))
    assert np.all(d1.data == 3)
    s, d1, d2 = _gr(op2, sizes)
    g = op2.Global(1, 0, dtype=np.uint32)
    op2.par_loop(op2.Kernel(K_INC, "k"), s, g(op2.INC), d1(op2.READ))
    total = int(np.sum(d1.data, dtype=np.int64))
    assert g.data[0] == total
    # repeated loops accumulate; resetting the data restarts
    op2.par_loop(op2.Kernel(K_INC, "k"), s, g(op2.INC), d1(op2.READ))
    assert g.data[0] == 2 * total
    g.data = 10
    op2.par_loop(op2.Kernel(K_INC, "k"), s, g(op2.INC), d1(op2.READ))
    assert g.data[0] == total + 10
    g2 = op2.Global(2, (0, 0), dtype=np.uint32)
    op2.par_loop(op2.Kernel(K2_INC, "k"), s, g2(op2.INC), d2(op2.READ))
    assert g2.data[0] == d2.data[:, 0].sum() and g2.data[1] == d2.data[:, 1].sum()


def sc_gr_minmax(op2, sizes=SIZES[0]):
    s, d1, d2 = _gr(op2, sizes)
    lo, hi = int(d1.data.min()), int(d1.data.max())
    for kern, acc, init, expect in ((K_MIN, op2.MIN, lo + 1, lo), (K_MIN, op2.MIN, lo - 1 + 1, lo),
                                    (K_MAX, op2.MAX, hi - 1, hi), (K_MAX, op2.MAX, hi + 1, hi + 1)):
        g = op2.Global(1, init, dtype=np.uint32)
        op2.par_loop(op2.Kernel(kern, "k"), s, g(acc), d1(op2.READ))
        assert g.data[0] == expect
    c0, c1 = d2.data[:, 0], d2.data[:, 1]
    g = op2.Global(2, (c0.min() + 1, c1.min() + 1), dtype=np.uint32)
    op2.par_loop(op2.Kernel(K2_MIN, "k"), s, g(op2.MIN), d2(op2.READ))
    assert g.data[0] == c0.min() and g.data[1] == c1.min()
    g = op2.Global(2, (c0.max() + 1, c1.max() + 1), dtype=np.uint32)
    op2.par_loop(op2.Kernel(K2_MAX, "k"), s, g(op2.MAX), d2(op2.READ))
    assert g.data[0] == c0.max() + 1 and g.data[1] == c1.max() + 1


def sc_gr_mixed_types(op2, sizes=SIZES[0]):
    s = op2.Set(sizes, "set")
    gu = op2.Global(1, [0], np.uint32, "g_uint32")
    gd = op2.Global(1, [0.0], np.float64, "g_double")
    k = "static void k(unsigned int* i, double* d) { *i += 1; *d += 1.0f; }"
    op2.par_loop(op2.Kernel(k, "k"), s, gu(op2.INC), gd(op2.INC))
    assert_allclose(gu.data[0], gd.data[0])
    assert gu.data[0] == s.size
    g = op2.Global(1, 0, dtype=np.uint32)
    op2.par_loop(op2.Kernel("static void k(unsigned int* g) { *g += 1; }", "k"), s, g(op2.INC))
    assert g.data[0] == s.size


# ------------------------------------------------------------------------
# test/unit/test_direct_loop.py:68-233 (direct WRITE/RW/INC + Global)
def sc_direct(op2):
    n = NELEMS
    elems = op2.Set(n, "elems")
    x = op2.Dat(op2.DataSet(elems, 1), np.arange(n, dtype=np.uint32), np.uint32)
    y = op2.Dat(op2.DataSet(elems, 2), np.array([np.arange(n)] * 2, dtype=np.uint32).T.copy(),
                np.uint32)
    op2.par_loop(op2.Kernel("static void k(unsigned int *x) { *x = 42; }", "k"), elems,
                 x(op2.WRITE))
    assert np.all(x.data == 42)
    op2.par_loop(op2.Kernel("static void k(unsigned int *x) { *x = *x + 1; }", "k"), elems,
                 x(op2.RW))
    assert np.all(x.data == 43)
    g = op2.Global(1, 0, np.uint32, "g")
    op2.par_loop(op2.Kernel("static void k(unsigned int *x, unsigned int *g) { *g += *x; }", "k"),
                 elems, x(op2.READ), g(op2.INC))
    assert g.data[0] == 43 * n
    op2.par_loop(op2.Kernel("static void k(unsigned int *y) { y[0] = 42; y[1] = 43; }", "k"),
                 elems, y(op2.WRITE))
    assert np.all(y.data[:, 0] == 42) and np.all(y.data[:, 1] == 43)
    op2.par_loop(op2.Kernel("static void k(unsigned int *y) { y[0] += 1; y[1] += 1; }", "k"),
                 elems, y(op2.INC))
    assert np.all(y.data[:, 0] == 43) and np.all(y.data[:, 1] == 44)


# ------------------------------------------------------------------------
# test/unit/test_indirect_loop.py:277-313, 316-468 (permuted / composed maps)
def sc_permuted_map(op2):
    fromset, toset = op2.Set(1), op2.Set(4)
    d1 = op2.Dat(op2.DataSet(toset, 1), dtype=np.int32)
    d2 = op2.Dat(op2.DataSet(toset, 1), dtype=np.int32)
    d1.data[:] = np.arange(4, dtype=np.int32)
    k = op2.Kernel("""
    void copy(int *to, const int * restrict from) {
        for (int i = 0; i < 4; i++) { to[i] = from[i]; }
    }""", "copy")
    m1 = op2.Map(fromset, toset, 4, values=[1, 2, 3, 0])
    perm = [3, 2, 0, 1]
    m2 = op2.PermutedMap(m1, perm)
    op2.par_loop(k, fromset, d2(op2.WRITE, m2), d1(op2.READ, m1))
    vals = np.array([[1, 2, 3, 0]])
    expect = np.empty(4, dtype=np.int32)
    expect[vals[..., perm]] = np.arange(4)[vals]
    assert np.all(d1.data == np.arange(4)) and np.all(d2.data == expect)


def sc_permuted_map_both(op2):
    """Both arguments through different permutations of one map
    (test/unit/test_indirect_loop.py:296-313)."""
    fromset, toset = op2.Set(1), op2.Set(4)
    d1 = op2.Dat(op2.DataSet(toset, 1), dtype=np.int32)
    d2 = op2.Dat(op2.DataSet(toset, 1), dtype=np.int32)
    d1.data[:] = np.arange(4, dtype=np.int32)
    k = op2.Kernel("""
    void copy(int *to, const int * restrict from) {
        for (int i = 0; i < 4; i++) { to[i] = from[i]; }
    }""", "copy")
    m1 = op2.Map(fromset, toset, 4, values=[0, 2, 1, 3])
    p2, p3 = [3, 2, 1, 0], [0, 2, 3, 1]
    m2 = op2.PermutedMap(m1, p2)
    m3 = op2.PermutedMap(m1, p3)
    op2.par_loop(k, fromset, d2(op2.WRITE, m2), d1(op2.READ, m3))
    vals = np.array([[0, 2, 1, 3]])
    expect = np.empty(4, dtype=np.int32)
    expect[vals[..., p2]] = np.arange(4, dtype=np.int32)[vals[..., p3]]
    assert np.all(d1.data == np.arange(4)) and np.all(d2.data == expect)


def sc_composed_two_maps(op2, permuted=False):
    setB, nodesetB = op2.Set(3), op2.Set(6)
    datB = op2.Dat(op2.DataSet(nodesetB, 1), dtype=np.float64)
    mapB = op2.Map(setB, nodesetB, 2, values=[[0, 1], [2, 3], [4, 5]])
    setA, nodesetA = op2.Set(5), op2.Set(8)
    datA = op2.Dat(op2.DataSet(nodesetA, 1), dtype=np.float64)
    datA.data[:] = np.array([.0, .1, .2, .3, .4, .5, .6, .7])
    mapA0 = op2.Map(setA, nodesetA, 2, values=[[0, 1], [2, 3], [4, 5], [6, 7], [0, 1]])
    if permuted:
        mapA0 = op2.PermutedMap(mapA0, [1, 0])
    mapA1 = op2.Map(setB, setA, 1, values=[3, 1, 2])
    mapA = op2.ComposedMap(mapA0, mapA1)
    k = op2.Kernel("""
    void copy(double *to, const double * restrict from) {
        for (int i = 0; i < 2; ++i) { to[i] = from[i]; }
    }""", "copy")
    op2.par_loop(k, setB, datB(op2.WRITE, mapB), datA(op2.READ, mapA))
    expect = [.7, .6, .3, .2, .5, .4] if permuted else [.6, .7, .2, .3, .4, .5]
    assert np.all(datB.data == np.array(expect))


def sc_composed_three_maps(op2, nested="none", subset=False):
    setC, nodesetC = op2.Set(2), op2.Set(4)
    datC = op2.Dat(op2.DataSet(nodesetC, 1), dtype=np.float64)
    mapC = op2.Map(setC, nodesetC, 2, values=[[0, 1], [2, 3]])
    setB, setA, nodesetA = op2.Set(3), op2.Set(5), op2.Set(8)
    datA = op2.Dat(op2.DataSet(nodesetA, 1), dtype=np.float64)
    datA.data[:] = np.array([.0, .1, .2, .3, .4, .5, .6, .7])
    mapA0 = op2.Map(setA, nodesetA, 2, values=[[0, 1], [2, 3], [4, 5], [6, 7], [0, 1]])
    mapA1 = op2.Map(setB, setA, 1, values=[3, 1, 2])
    mapA2 = op2.Map(setC, setB, 1, values=[2, 0])
    if nested == "none":
        mapA = op2.ComposedMap(mapA0, mapA1, mapA2)
    elif nested == "first":
        mapA = op2.ComposedMap(op2.ComposedMap(mapA0, mapA1), mapA2)
    else:
        mapA = op2.ComposedMap(mapA0, op2.ComposedMap(mapA1, mapA2))
    k = op2.Kernel("""
    void copy(double *to, const double * restrict from) {
        for (int i = 0; i < 2; ++i) { to[i] = from[i]; }
    }""", "copy")
    it = op2.Subset(setC, np.array([1], dtype=np.int32)) if subset else setC
    op2.par_loop(k, it, datC(op2.WRITE, mapC), datA(op2.READ, mapA))
    expect = [.0, .0, .6, .7] if subset else [.4, .5, .6, .7]
    assert np.all(datC.data == np.array(expect))


# ------------------------------------------------------------------------
# test/unit/test_subset.py (direct and indirect loops over subsets)
def sc_subset_direct(op2):
    iterset = op2.Set(NELEMS)
    indices = np.arange(0, NELEMS, 2, dtype=np.int32)
    ss = op2.Subset(iterset, indices)
    d = op2.Dat(iterset ** 1, np.ones(NELEMS), np.uint32)
    op2.par_loop(op2.Kernel("static void inc(unsigned int* v) { *v += 1; }", "inc"), ss,
                 d(op2.RW))
    assert int(np.sum(d.data, dtype=np.int64)) == NELEMS + NELEMS // 2


def sc_subset_indirect(op2):
    iterset = op2.Set(NELEMS)
    unitset = op2.Set(1)
    u = op2.Dat(unitset, np.array([0], dtype=np.uint32), np.uint32)
    m = op2.Map(iterset, unitset, 1, np.zeros(NELEMS, dtype=np.int32))
    ss = op2.Subset(iterset, np.arange(1, NELEMS, 3, dtype=np.int32))
    op2.par_loop(op2.Kernel("static void inc(unsigned int* x) { (*x) += 1; }", "inc"), ss,
                 u(op2.INC, m))
    assert u.data[0] == len(range(1, NELEMS, 3))


# ------------------------------------------------------------------------
# test/unit/test_extrusion.py:334-444 (constant layers, offsets)
EXT_NELEMS, EXT_LAYERS = 32, 11


def _ext(op2):
    nelems, layers = EXT_NELEMS, EXT_LAYERS
    wedges = layers - 1
    nnodes = nelems + 2
    elements = op2.ExtrudedSet(op2.Set(nelems), layers)
    node_set = op2.Set(nnodes * layers, "nodes1")
    elem_set = op2.Set(nelems * wedges, "elems1")
    # coordinate map: 3 base nodes (i, i+1, i+2) x 2 levels, column-numbered nodes
    base = np.array([[i, i + 1, i + 2] for i in range(nelems)])
    cmap = np.concatenate([base * layers, base * layers + 1], axis=1)
    cmap = cmap[:, [0, 3, 1, 4, 2, 5]].astype(np.int32)
    coords_map = op2.Map(elements, node_set, 6, cmap, "elem_dofs",
                         np.ones(6, dtype=np.int32))
    field_map = op2.Map(elements, elem_set, 1, (np.arange(nelems) * wedges).astype(np.int32),
                        "elem_elem", np.ones(1, dtype=np.int32))
    cd = np.zeros((nnodes, layers, 2))
    k = np.arange(nnodes)
    cd[:, :, 0] = (k // 2)[:, None]
    cd[:, :, 1] = (k % 2)[:, None]
    dat_coords = op2.Dat(op2.DataSet(node_set, 2), cd.reshape(-1, 2), np.float64, "coords")
    dat_field = op2.Dat(op2.DataSet(elem_set, 1), np.ones(nelems * wedges), np.float64, "field")
    return elements, node_set, elem_set, coords_map, field_map, dat_coords, dat_field


def sc_extrusion_volume(op2):
    elements, node_set, elem_set, coords_map, field_map, dat_coords, dat_field = _ext(op2)
    g = op2.Global(1, data=0.0, name="g")
    mass = op2.Kernel("""
static void comp_vol(double A[1], double x[6][2], double y[1])
{
    double abs = x[0][0]*(x[2][1]-x[4][1])+x[2][0]*(x[4][1]-x[0][1])+x[4][0]*(x[0][1]-x[2][1]);
    if (abs < 0)
      abs = abs * (-1.0);
    A[0]+=0.5*abs*0.1 * y[0];
}""", "comp_vol")
    op2.par_loop(mass, elements, g(op2.INC), dat_coords(op2.READ, coords_map),
                 dat_field(op2.READ, field_map))
    # The reference test truncates int(g); its value, 320 contributions of 0.05,
    # is 16 only up to rounding, so compare with a tolerance instead (a
    # parallel reduction sums in another order than the sequential loop).
    assert abs(g.data[0] - (EXT_LAYERS - 1) * 0.1 * (EXT_NELEMS // 2)) <= 1e-12
    return float(g.data[0])


def sc_extrusion_fields(op2):
    """test_extruded_nbytes, test_write_data_field, test_write_data_coords,
    test_read_coord_neighbours_write_to_field (test/unit/test_extrusion.py:
    358-426)."""
    elements, node_set, elem_set, coords_map, field_map, dat_coords, dat_field = _ext(op2)
    wedges = EXT_LAYERS - 1
    if hasattr(dat_field, "nbytes"):
        assert dat_field.nbytes == EXT_NELEMS * wedges * 8
    dat_f = op2.Dat(op2.DataSet(elem_set, 1), -np.ones(EXT_NELEMS * wedges), np.float64, "f")
    op2.par_loop(op2.Kernel("static void wo(double* x) { x[0] = 42.0; }\n", "wo"), elements,
                 dat_f(op2.WRITE, field_map))
    assert np.all(dat_f.data == 42)
    dat_c = op2.Dat(op2.DataSet(node_set, 2), np.zeros(((EXT_NELEMS + 2) * EXT_LAYERS, 2)),
                    np.float64, "c")
    op2.par_loop(op2.Kernel("""static void wo_c(double x[6][2]) {
       for (int i = 0; i < 6; ++i) { x[i][0] = 42.0; x[i][1] = 42.0; } }""", "wo_c"), elements,
                 dat_c(op2.WRITE, coords_map))
    assert np.all(dat_c.data == 42)
    op2.par_loop(op2.Kernel("""static void wtf(double* y, double x[6][2]) {
       double sum = 0.0;
       for (int i=0; i<6; i++) sum += x[i][0] + x[i][1];
       y[0] = sum; }""", "wtf"), elements, dat_f(op2.WRITE, field_map),
                 dat_coords(op2.READ, coords_map))
    assert np.all(dat_f.data >= 0)
    return dat_f.data.copy()


def sc_extrusion_direct_inc(op2):
    iterset = op2.Set(EXT_NELEMS)
    dat = op2.Dat(op2.DataSet(iterset, 1))
    xtr = op2.ExtrudedSet(iterset, 10)
    dat.data[:] = 0
    op2.par_loop(op2.Kernel("static void k(double *x) { *x += 1.0; }", "k"), xtr, dat(op2.INC))
    assert np.allclose(dat.data[:], 9.0)


def sc_extrusion_layer_arg(op2):
    elements, node_set, elem_set, coords_map, field_map, dat_coords, dat_field = _ext(op2)
    dat_f = op2.Dat(op2.DataSet(elem_set, 1), -np.ones(EXT_NELEMS * (EXT_LAYERS - 1)),
                    np.float64, "f")
    k = "static void blah(double* x, int layer_arg){ x[0] = layer_arg; }"
    op2.par_loop(op2.Kernel(k, "blah"), elements, dat_f(op2.WRITE, field_map), pass_layer_arg=True)
    ref = np.tile(np.arange(EXT_LAYERS - 1), EXT_NELEMS)
    assert np.all(dat_f.data == ref)


def sc_extrusion_write_coords(op2, sequential=True):
    elements, node_set, elem_set, coords_map, field_map, dat_coords, dat_field = _ext(op2)
    dat_c = op2.Dat(op2.DataSet(node_set, 2), np.zeros(((EXT_NELEMS + 2) * EXT_LAYERS, 2)),
                    np.float64, "c")
    k = """static void inc(double y[6][2], double x[6][2]) {
       for (int i=0; i<6; i++){ if (y[i][0] == 0){ y[i][0] += 1; y[i][1] += 1; } } }"""
    op2.par_loop(op2.Kernel(k, "inc"), elements, dat_c(op2.RW, coords_map),
                 dat_coords(op2.READ, coords_map))
    if sequential:
        assert np.sum(dat_c.data) == (EXT_NELEMS + 2) * EXT_LAYERS * 2
    else:
        # RW through a map onto entities shared by concurrently executing
        # cells is a write conflict the user owns (pyop2/types/access.py:21-24):
        # a cell may read one component before and the other after a
        # neighbour's update, then write back the stale second component.
        # What a parallel run guarantees is that every node was reached
        # (every write-back of a node stores first component 1) and that the
        # second component is 0 or 1.
        d = dat_c.data
        assert np.all(d[:, 0] == 1) and np.all((d[:, 1] == 0) | (d[:, 1] == 1))


# ------------------------------------------------------------------------
# test/unit/test_matrices.py:54-131, 461-699 (2 triangles on 4 nodes)
ELEM_NODE = np.asarray([0, 1, 3, 2, 3, 1], dtype=np.uint32)
COORDS = np.asarray([(0.0, 0.0), (2.0, 0.0), (1.0, 1.0), (0.0, 1.5)])
EXPECTED_MASS = np.asarray([(0.25, 0.125, 0.0, 0.125),
                            (0.125, 0.291667, 0.0208333, 0.145833),
                            (0.0, 0.0208333, 0.0416667, 0.0208333),
                            (0.125, 0.145833, 0.0208333, 0.291667)])
EXPECTED_RHS = np.asarray([0.9999999523522115, 1.3541666031724144, 0.2499999883507239,
                           1.6458332580869566])

_QUAD = """
  double CG1[3][6] = { {  0.09157621, 0.09157621, 0.81684757, 0.44594849, 0.44594849, 0.10810302 },
                       {  0.09157621, 0.81684757, 0.09157621, 0.44594849, 0.10810302, 0.44594849 },
                       {  0.81684757, 0.09157621, 0.09157621, 0.10810302, 0.44594849, 0.44594849 } };
  double d_CG1[3][2] = { { 1., 0. }, { 0., 1. }, { -1., -1. } };
  double w[6] = {  0.05497587, 0.05497587, 0.05497587, 0.11169079, 0.11169079, 0.11169079 };
  double c_q0[2][2];
  for (int a = 0; a < 2; a++) for (int b = 0; b < 2; b++) {
    c_q0[a][b] = 0.0;
    for (int r = 0; r < 3; r++) c_q0[a][b] += c0[r][a] * d_CG1[r][b];
  }
  const double det = c_q0[0][0] * c_q0[1][1] - c_q0[0][1] * c_q0[1][0];
"""
MASS = ("static void mass(double localTensor[3][3], double c0[3][2]) {" + _QUAD + """
  for (int g = 0; g < 6; g++)
    for (int i = 0; i < 3; ++i)
      for (int j = 0; j < 3; ++j)
        localTensor[i][j] += CG1[i][g] * CG1[j][g] * det * w[g];
}""")
RHS = ("static void rhs(double* localTensor, double c0[3][2], double* c1) {" + _QUAD + """
  for (int g = 0; g < 6; g++) {
    double f = 0.0;
    for (int r = 0; r < 3; r++) f += c1[r] * CG1[r][g];
    for (int i = 0; i < 3; ++i) localTensor[i] += CG1[i][g] * f * det * w[g];
  }
}""")


def _mat_fixture(op2):
    nodes = op2.Set(4, "nodes")
    elements = op2.Set(2, "elements")
    dnodes = op2.DataSet(nodes, 1, "dnodes")
    dvnodes = op2.DataSet(nodes, 2, "dvnodes")
    elem_node = op2.Map(elements, nodes, 3, ELEM_NODE, "elem_node")
    coords = op2.Dat(dvnodes, COORDS, np.float64, "coords")
    return nodes, elements, dnodes, dvnodes, elem_node, coords


def sc_mass_matrix(op2):
    nodes, elements, dnodes, dvnodes, elem_node, coords = _mat_fixture(op2)
    sp = op2.Sparsity((dnodes, dnodes), [(elem_node, elem_node, None)])
    mat = op2.Mat(sp)
    mat.zero()
    op2.par_loop(op2.Kernel(MASS, "mass"), elements, mat(op2.INC, (elem_node, elem_node)),
                 coords(op2.READ, elem_node))
    mat.assemble()
    assert_allclose(mat.values, EXPECTED_MASS, 1e-5)
    return mat.values


def sc_rhs(op2):
    nodes, elements, dnodes, dvnodes, elem_node, coords = _mat_fixture(op2)
    f = op2.Dat(dnodes, np.asarray([1.0, 2.0, 3.0, 4.0]), np.float64, "f")
    b = op2.Dat(dnodes, np.zeros(4), np.float64, "b")
    op2.par_loop(op2.Kernel(RHS, "rhs"), elements, b(op2.INC, elem_node),
                 coords(op2.READ, elem_node), f(op2.READ, elem_node))
    assert_allclose(b.data, EXPECTED_RHS, 1e-7)
    return b.data.copy()


def sc_set_matrix(op2):
    """INC ones, then WRITE ones (test/unit/test_matrices.py:679-696)."""
    nodes, elements, dnodes, dvnodes, elem_node, coords = _mat_fixture(op2)
    mat = op2.Mat(op2.Sparsity((dnodes, dnodes), [(elem_node, elem_node, None)]))
    g = op2.Global(1, 1.0, np.float64, "g")
    kinc = """static void inc(double entry[3][3], double* g) {
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) entry[i][j] += g[0]; }"""
    kset = """static void set(double entry[3][3], double* g) {
      for (int i = 0; i < 3; i++) for (int j = 0; j < 3; j++) entry[i][j] = g[0]; }"""
    mat.zero()
    op2.par_loop(op2.Kernel(kinc, "inc"), elements, mat(op2.INC, (elem_node, elem_node)),
                 g(op2.READ))
    mat.assemble()
    assert mat.values.sum() == 3 * 3 * 2
    op2.par_loop(op2.Kernel(kset, "set"), elements, mat(op2.WRITE, (elem_node, elem_node)),
                 g(op2.READ))
    mat.assemble()
    # INSERT of ones: the two elements share an edge (4 shared entries), so
    # 14 distinct entries hold 1
    assert mat.values.sum() == (3 * 3 - 2) * 2


def sc_vector_mass_matrix(op2):
    """2-component mass matrix, BAIJ with 2x2 blocks
    (test/unit/test_matrices.py:467-482 expected_vector_matrix)."""
    nodes, elements, dnodes, dvnodes, elem_node, coords = _mat_fixture(op2)
    vmat = op2.Mat(op2.Sparsity((dvnodes, dvnodes), [(elem_node, elem_node, None)]))
    k = ("static void mass_vec(double localTensor[6][6], double c0[3][2]) {" + _QUAD + """
  for (int g = 0; g < 6; g++)
    for (int i = 0; i < 3; ++i) for (int j = 0; j < 3; ++j) {
      const double v = CG1[i][g] * CG1[j][g] * det * w[g];
      localTensor[2 * i][2 * j] += v; localTensor[2 * i + 1][2 * j + 1] += v; }
}""")
    op2.par_loop(op2.Kernel(k, "mass_vec"), elements, vmat(op2.INC, (elem_node, elem_node)),
                 coords(op2.READ, elem_node))
    vmat.assemble()
    expect = np.kron(EXPECTED_MASS, np.eye(2))
    assert_allclose(vmat.values, expect, 1e-5)
    return vmat.values


def sc_sparsity_nnz(op2):
    """test/unit/test_matrices.py:555-566."""
    s, d = op2.Set(1), op2.Set(4)
    m = op2.Map(s, d, 2, [1, 3])
    d2 = op2.Set(4)
    m2 = op2.Map(s, d2, 3, [1, 2, 3])
    sp = op2.Sparsity((d ** 1, d ** 1), [(m, m, None)])
    sp2 = op2.Sparsity((d ** 1, d2 ** 1), [(m, m2, None)])
    assert np.all(sp.nnz == [1, 2, 1, 2])
    assert np.all(sp2.nnz == [0, 3, 0, 3])


def sc_sparsity_blockwise(op2):
    """Off-diagonal blocks of test/unit/test_matrices.py:944-981, built as
    stand-alone sparsities (composed maps with a negative entry)."""
    setA, nodesetA = op2.Set(3), op2.Set(4)
    setB, nodesetB = op2.Set(2), op2.Set(3)
    mapA = op2.Map(setA, nodesetA, 2, values=[[0, 1], [1, 2], [2, 3]])
    mapB = op2.Map(setB, nodesetB, 2, values=[[0, 1], [1, 2]])
    mapBA = op2.Map(setB, setA, 1, values=[1, 2])
    mapAB = op2.Map(setA, setB, 1, values=[-1, 0, 1])
    s01 = op2.Sparsity((nodesetA ** 1, nodesetB ** 1),
                       [(mapA, op2.ComposedMap(mapB, mapAB), None)], diagonal_block=False)
    s10 = op2.Sparsity((nodesetB ** 1, nodesetA ** 1),
                       [(mapB, op2.ComposedMap(mapA, mapBA), None)], diagonal_block=False)
    assert np.all(s01.nnz == [0, 2, 3, 2])
    assert np.all(s10.nnz == [2, 3, 2])


def sc_extruded_sparsity(op2):
    """Extruded prism pattern (test/unit/test_matrices.py:58 xtr_elem_node_map
    with 11 layers, offsets 1)."""
    layers = 11
    xtr_elements = op2.ExtrudedSet(op2.Set(2), layers)
    xtr_nodes = op2.Set(4 * layers)
    vals = np.asarray([0, 1, 11, 12, 33, 34, 22, 23, 33, 34, 11, 12], dtype=np.int32)
    m = op2.Map(xtr_elements, xtr_nodes, 6, vals, "xtr_elem_node", np.ones(6, dtype=np.int32))
    sp = op2.Sparsity((xtr_nodes ** 1, xtr_nodes ** 1), [(m, m, None)])
    return np.asarray(sp.nnz).copy()


# ------------------------------------------------------------------------
# test/unit/test_indirect_loop.py:365-468 (composed map over extruded sets)
def sc_composed_map_extrusion(op2, variable=False, subset=False):
    arity = 3
    if variable:
        setC = op2.ExtrudedSet(op2.Set(2), [[1, 3], [0, 3]])
        nodesetC = op2.Set(8)
        mapC = op2.Map(setC, nodesetC, arity, values=[[5, 6, 7], [0, 1, 2]], offset=[2, 2, 2])
        setA = op2.ExtrudedSet(op2.Set(3), [[0, 3], [1, 3], [0, 3]])
        nodesetA = op2.Set(13)
        datA = op2.Dat(op2.DataSet(nodesetA, 1), np.arange(13, dtype=np.float64))
        mapA0 = op2.Map(setA, nodesetA, arity, values=[[8, 9, 10], [5, 6, 7], [0, 1, 2]],
                        offset=[2, 2, 2])
        expected = [0., 1., 2., 3., 4., 0., 0., 0.] if subset else [0., 1., 2., 3., 4., 5., 6., 7.]
    else:
        setC = op2.ExtrudedSet(op2.Set(2), 3)
        nodesetC = op2.Set(10)
        mapC = op2.Map(setC, nodesetC, arity, values=[[5, 6, 7], [0, 1, 2]], offset=[2, 2, 2])
        setA = op2.ExtrudedSet(op2.Set(3), 3)
        nodesetA = op2.Set(15)
        datA = op2.Dat(op2.DataSet(nodesetA, 1), np.arange(15, dtype=np.float64))
        mapA0 = op2.Map(setA, nodesetA, arity, values=[[10, 11, 12], [5, 6, 7], [0, 1, 2]],
                        offset=[2, 2, 2])
        expected = ([0., 1., 2., 3., 4., 0., 0., 0., 0., 0.] if subset
                    else [0., 1., 2., 3., 4., 5., 6., 7., 8., 9.])
    datC = op2.Dat(op2.DataSet(nodesetC, 1), dtype=np.float64)
    mapA1 = op2.Map(setC, setA, 1, values=[1, 2])
    mapA = op2.ComposedMap(mapA0, mapA1)
    k = op2.Kernel("""
    void copy(double *to, const double * restrict from) {
        for (int i = 0; i < 3; ++i) { to[i] = from[i]; }
    }""", "copy")
    it = op2.Subset(setC, np.array([1], dtype=np.int32)) if subset else setC
    op2.par_loop(k, it, datC(op2.WRITE, mapC), datA(op2.READ, mapA))
    assert np.all(np.asarray(datC.data) == np.array(expected))


def sc_extruded_regions(op2, region, periodic=False, variable=False):
    """INC through an offset map under each iteration region, with the layer
    argument; returns the result for cross-implementation comparison."""
    nb = 5
    if variable:
        layers = np.array([[0, 5], [1, 6], [0, 3], [2, 6], [0, 6]], dtype=np.int32)
    else:
        layers = 6
    base = op2.Set(nb)
    ext = op2.ExtrudedSet(base, layers, extruded_periodic=periodic) if periodic else \
        op2.ExtrudedSet(base, layers)
    L = 6
    nodes = op2.Set((nb + 1) * L)
    vals = np.array([[i * L, (i + 1) * L] for i in range(nb)], dtype=np.int32)
    kw = dict(offset=[1, 1])
    if periodic:
        kw["offset_quotient"] = [0, 1]
    m = op2.Map(ext, nodes, 2, vals, **kw)
    d = op2.Dat(nodes, np.zeros((nb + 1) * L))
    nf = 2 if region == op2.ON_INTERIOR_FACETS else 1
    k = op2.Kernel("static void k(double *x, int layer) { for (int i = 0; i < %d; ++i) "
                   "x[i] += (i + 1) * (layer + 1); }" % (2 * nf), "k")
    op2.par_loop(k, ext, d(op2.INC, m), iteration_region=region, pass_layer_arg=True)
    return np.asarray(d.data).copy()


# ------------------------------------------------------------------------
# Mixed spaces: test/unit/test_indirect_loop.py:235-269 (TestMixedIndirectLoop)
def _mixed_indirect_fixture(op2, sizes=SIZES[0]):
    iterset = op2.Set(sizes, "iterset")
    indset = op2.Set(NELEMS, "indset")
    unitset = op2.Set(1, "unitset")
    mapd = np.arange(NELEMS)[::-1].astype(np.uint32)
    i2ind = op2.Map(iterset, indset, 1, mapd, "iterset2indset")
    i2unit = op2.Map(iterset, unitset, 1, np.zeros(NELEMS, dtype=np.uint32), "iterset2unitset")
    mset = op2.MixedSet((indset, unitset))
    return iterset, op2.MixedDat(mset), op2.MixedMap((i2ind, i2unit))


def sc_mixed_non_mixed_dat(op2, sizes=SIZES[0], itspace=False):
    """Increment into a MixedDat from a non-mixed Dat (both reference variants)."""
    iterset, mdat, mmap = _mixed_indirect_fixture(op2, sizes)
    d = op2.Dat(iterset, np.ones(NELEMS))
    if itspace:
        k = """static void inc(double *d, double *x) {
          for (int i=0; i<2; ++i) d[i] += x[0]; }"""
    else:
        k = "static void inc(double *d, double *x) { d[0] += x[0]; d[1] += x[0]; }"
    op2.par_loop(op2.Kernel(k, "inc"), iterset, mdat(op2.INC, mmap), d(op2.READ))
    assert np.all(mdat[0].data == 1.0) and mdat[1].data[0] == float(NELEMS)


# test/unit/test_matrices.py:500-530 (fixtures), 864-938 (TestMixedMatrices)
MIXED_OD = np.array([[1.0, 2.0, 0.0, 0.0],
                     [0.0, 4.0, 6.0, 0.0],
                     [0.0, 0.0, 9.0, 12.0]])
MIXED_LL = (np.diag([1.0, 8.0, 18.0, 16.0]) + np.diag([2.0, 6.0, 12.0], -1)
            + np.diag([2.0, 6.0, 12.0], 1))


def _mixed_mat_fixture(op2):
    elem, node = op2.Set(3), op2.Set(4)
    mset = op2.MixedSet((elem, node))
    rdata = lambda n: np.arange(1, n + 1, dtype=np.float64)
    mdat = op2.MixedDat([op2.Dat(s, rdata(s.size)) for s in mset])
    mmap = op2.MixedMap((op2.Map(elem, elem, 1, [0, 1, 2]),
                         op2.Map(elem, node, 2, [0, 1, 1, 2, 2, 3])))
    return elem, node, mset, mdat, mmap, rdata


def sc_mixed_mat(op2, nest=True):
    """Assemble into a matrix on a mixed sparsity (block values asserted by
    test_assemble_mixed_mat); ``nest`` selects nested or monolithic."""
    elem, node, mset, mdat, mmap, rdata = _mixed_mat_fixture(op2)
    blocks = {(i, j): [(rm, cm, None)] for i, rm in enumerate(mmap) for j, cm in enumerate(mmap)}
    sp = op2.Sparsity((mset ** 1, mset ** 1), blocks, nest=nest)
    mat = op2.Mat(sp)
    k = """static void addone_mat(double v[9], double d[3]) {
        for (int i = 0; i < 3; i++)
           for (int j = 0; j < 3; j++)
              v[i*3 + j] += d[i]*d[j];
    }"""
    op2.par_loop(op2.Kernel(k, "addone_mat"), elem, mat(op2.INC, (mmap, mmap)),
                 mdat(op2.READ, mmap))
    mat.assemble()
    eps = 1.e-12
    assert_allclose(mat[0, 0].values, np.diag([1.0, 4.0, 9.0]), eps)
    assert_allclose(mat[0, 1].values, MIXED_OD, eps)
    assert_allclose(mat[1, 0].values, MIXED_OD.T, eps)
    assert_allclose(mat[1, 1].values, MIXED_LL, eps)
    whole = np.block([[np.diag([1.0, 4.0, 9.0]), MIXED_OD], [MIXED_OD.T, MIXED_LL]])
    assert_allclose(mat.values, whole, eps)
    return sp, mat


def sc_mixed_rhs(op2):
    """test_assemble_mixed_rhs."""
    elem, node, mset, mdat, mmap, rdata = _mixed_mat_fixture(op2)
    dat = op2.MixedDat(mset)
    k = """static void addone_rhs(double v[3], double d[3]) {
      for (int i=0; i<3; ++i) v[i] += d[i]; }"""
    op2.par_loop(op2.Kernel(k, "addone_rhs"), elem, dat(op2.INC, mmap), mdat(op2.READ, mmap))
    eps = 1.e-12
    assert_allclose(dat[0].data_ro, rdata(3), eps)
    assert_allclose(dat[1].data_ro, [1.0, 4.0, 6.0, 4.0], eps)


def sc_mixed_rhs_vector(op2):
    """test_assemble_mixed_rhs_vector: dim-2 components."""
    elem, node, mset, mdat, mmap, rdata = _mixed_mat_fixture(op2)
    mvdat = op2.MixedDat([op2.Dat(s ** 2, np.stack([rdata(s.size), rdata(s.size)], 1))
                          for s in mset])
    dat = op2.MixedDat(mset ** 2)
    k = """static void addone_rhs_vec(double v[6], double d[3][2]) {
      for (int i=0; i<3; ++i) { v[i*2+0] += d[i][0]; v[i*2+1] += d[i][1]; } }"""
    op2.par_loop(op2.Kernel(k, "addone_rhs_vec"), elem, dat(op2.INC, mmap),
                 mvdat(op2.READ, mmap))
    eps = 1.e-12
    exp = np.kron(np.array([1.0, 4.0, 6.0, 4.0])[:, None], np.ones(2))
    assert_allclose(dat[0].data_ro, np.kron(rdata(3)[:, None], np.ones(2)), eps)
    assert_allclose(dat[1].data_ro, exp, eps)


# ------------------------------------------------------------------------
# A larger mixed problem for oracle-vs-GPU parity: P1 (vertices, dim 2) x
# P0 (cells, dim 1) on the jittered split-square mesh; one mixed element
# matrix (7 x 7) INC'd into a mixed Mat, and its action on a mixed vector
# INC'd into a MixedDat.
MIXED_P1P0 = """
static void mixed_p1p0(double A[7][7], double b[7], const double *u, const double X[3][2])
{
  const double det = fabs((X[1][0] - X[0][0]) * (X[2][1] - X[0][1])
                          - (X[2][0] - X[0][0]) * (X[1][1] - X[0][1]));
  for (int i = 0; i < 7; ++i)
    for (int j = 0; j < 7; ++j)
      A[i][j] += det * (1.0 + 0.1 * i + 0.01 * j + (i == j ? 2.0 : 0.0)) * (X[i % 3][0] + 0.5);
  for (int i = 0; i < 7; ++i) {
    double s = 0.0;
    for (int j = 0; j < 7; ++j) s += A[i][j] * u[j];
    b[i] += s;
  }
}
"""


def sc_mixed_p1p0(op2, n=16, nest=True, seed=3):
    from pyop2_gb300.meshes import unit_square_tris
    coords, tris = unit_square_tris(n, seed=seed)
    V, C = coords.shape[0], tris.shape[0]
    verts, cells = op2.Set(V, "verts"), op2.Set(C, "cells")
    c2v = op2.Map(cells, verts, 3, tris, "c2v")
    c2c = op2.Map(cells, cells, 1, np.arange(C, dtype=np.int32), "c2c")
    mset = op2.MixedSet((verts, cells))
    mdset = op2.MixedDataSet(mset, (2, 1))
    mmap = op2.MixedMap((c2v, c2c))
    X = op2.Dat(verts ** 2, coords, np.float64, "X")
    rng = np.random.default_rng(seed)
    u = op2.MixedDat([op2.Dat(verts ** 2, rng.uniform(-1, 1, (V, 2))),
                      op2.Dat(cells, rng.uniform(-1, 1, C))])
    b = op2.MixedDat(mdset)
    blocks = {(i, j): [(rm, cm, None)] for i, rm in enumerate(mmap) for j, cm in enumerate(mmap)}
    A = op2.Mat(op2.Sparsity((mdset, mdset), blocks, nest=nest))
    op2.par_loop(op2.Kernel(MIXED_P1P0, "mixed_p1p0"), cells, A(op2.INC, (mmap, mmap)),
                 b(op2.INC, mmap), u(op2.READ, mmap), X(op2.READ, c2v))
    A.assemble()
    return A, b
