"""Colouring plans are cached on the iteration set per tuple of written maps.
A map that is freed and replaced by another (which may reuse its id()) must
get a plan of its own: a stale plan would let two cells of one colour share
a target, a silent race under coloured execution."""
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

K = "static void k(double *y, const double *w) { y[0] += w[0]; y[1] += w[0]; }"


def _loop(op2, cells, verts, values, w, y):
    m = op2.Map(cells, verts, 2, values)
    return m, op2.ParLoop(op2.Kernel(K, "k"), cells, y(op2.INC, m), w(op2.READ))


def test_plan_of_a_freed_map_is_not_reused(gpu_op2):
    from pyop2_gb300.parloop import colour_plan
    op2 = gpu_op2
    n, nv = 4096, 4097
    cells, verts = op2.Set(n), op2.Set(nv)
    w = op2.Dat(cells, np.ones(n))
    y = op2.Dat(verts, np.zeros(nv))
    # a chain: cell i touches vertices i, i+1 (two colours suffice)
    chain = np.stack([np.arange(n), np.arange(n) + 1], axis=1).astype(np.int32)
    m, lp = _loop(op2, cells, verts, chain, w, y)
    p1 = colour_plan(lp)
    assert p1 is not None and p1.validate([m])
    del lp, m
    gc.collect()
    rng = np.random.default_rng(0)
    for _ in range(8):
        # other connectivity on the same iteration set: every cell also hits
        # a random vertex, so the chain's 2-colouring is no longer valid
        vals = np.stack([np.arange(n), rng.integers(0, nv, n)], axis=1).astype(np.int32)
        m2, lp2 = _loop(op2, cells, verts, vals, w, y)
        p2 = colour_plan(lp2)
        assert p2 is not None and p2 is not p1
        assert p2.validate([m2])
        # coloured execution with the new plan equals the atomic result
        from pyop2_gb300.configuration import configuration
        old = configuration["scatter"]
        try:
            y.zero()
            configuration["scatter"] = "colour"
            op2.par_loop(op2.Kernel(K, "k"), cells, y(op2.INC, m2), w(op2.READ))
            got = y.data_ro.copy()
        finally:
            configuration["scatter"] = old
        ref = np.zeros(nv)
        np.add.at(ref, vals[:, 0], 1.0)
        np.add.at(ref, vals[:, 1], 1.0)
        assert np.array_equal(got, ref)
        del lp2, m2
        gc.collect()
