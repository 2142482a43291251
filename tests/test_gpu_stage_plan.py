"""Staging plans (op2g_stage_plan_count / _fill) against a numpy restatement
of the local renumbering of the historical OP2 execution plan
(doc/sphinx/source/plan.rst:21-39): per partition of `block` iterations, the
sorted distinct non-negative map values, and per map entry the position of
its value in that list (0xFFFF for a negative entry)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def plan_model(vals, block):
    """Per partition: the padded segment, the sorted distinct targets, the
    first slot of each and the number of valid entries, and every entry's
    slot (its rank among the partition's valid entries sorted by (target,
    position))."""
    n, ar = vals.shape
    off, num, ind, runs = [0], [], [], []
    loc = np.full(n * ar, 0xFFFF, dtype=np.int64)
    for c0 in range(0, n, block):
        v = vals[c0:c0 + block].reshape(-1)
        valid = np.nonzero(v >= 0)[0]
        order = valid[np.lexsort((valid, v[valid]))]       # by target, then position
        loc[c0 * ar + order] = np.arange(len(order))
        u, first = np.unique(v[order], return_index=True)
        seg = (len(u) + 1 + 7) // 8 * 8
        ind.append((u, np.append(first, len(order)), seg))
        num.append(len(u))
        off.append(off[-1] + seg)
    return np.array(off), np.array(num), ind, loc


@pytest.mark.parametrize("n,arity,block,ntargets", [
    (1, 1, 32, 1), (1000, 3, 64, 50), (4097, 4, 512, 100000), (5000, 6, 96, 300),
    (3000, 2, 2048, 7)])
def test_plan_matches_model(gpu_op2, n, arity, block, ntargets):
    from pyop2_gb300.parloop import MapStagePlan
    op2 = gpu_op2
    rng = np.random.default_rng(n + arity)
    vals = rng.integers(0, ntargets, (n, arity)).astype(np.int32)
    vals[rng.random((n, arity)) < 0.05] = -1          # "no target" entries
    src, dst = op2.Set(n), op2.Set(ntargets)
    m = op2.Map(src, dst, arity, vals)
    p = MapStagePlan(m, block)
    off, num, segs, loc = plan_model(vals, block)
    assert np.array_equal(p.ind_off.cpu().numpy(), off)
    assert np.array_equal(p.ind_num.cpu().numpy()[:len(num)], num)
    assert p.total == off[-1]
    ind = p.ind_map.cpu().numpy()
    runs = p.run_off.cpu().numpy().astype(np.int64) & 0xFFFF
    for b, (u, first, seg) in enumerate(segs):
        assert np.array_equal(ind[off[b]:off[b] + len(u)], u)
        assert np.array_equal(runs[off[b]:off[b] + len(u) + 1], first)
    got = p.loc_map.cpu().numpy()[:n * arity].astype(np.int64) & 0xFFFF
    assert np.array_equal(got, loc)
    assert p.max_unique == int(np.max(num))


def test_staged_loop_equals_atomic_loop_with_negative_entries(gpu_op2):
    """A gather + INC loop through a map with -1 entries under the staged
    wrapper equals the same loop under atomics (integer values: exact)."""
    from pyop2_gb300.configuration import configuration
    op2 = gpu_op2
    rng = np.random.default_rng(5)
    n, nv = 20000, 3000
    vals = rng.integers(0, nv, (n, 3)).astype(np.int32)
    vals[rng.random((n, 3)) < 0.1] = -1
    cells, verts = op2.Set(n), op2.Set(nv)
    m = op2.Map(cells, verts, 3, vals)
    x = op2.Dat(verts ** 2, rng.integers(-9, 9, (nv, 2)).astype(np.float64))
    src = """static void k(double *y, const double *x, double *g) {
      for (int i = 0; i < 3; ++i) { y[i] += x[2 * i] + 2.0 * x[2 * i + 1]; g[0] += x[2 * i]; } }"""
    out = {}
    for sc in ("atomic", "staged"):
        y = op2.Dat(verts, np.zeros(nv))
        g = op2.Global(1, 0.0)
        old = configuration["scatter"]
        configuration["scatter"] = sc
        try:
            pl = op2.ParLoop(op2.Kernel(src, "k"), cells, y(op2.INC, m), x(op2.READ, m), g(op2.INC))
            pl.compute()
            pl.compute()
        finally:
            configuration["scatter"] = old
        out[sc] = (y.data_ro.copy(), g.data_ro[0])
    assert np.array_equal(out["atomic"][0], out["staged"][0])
    assert out["atomic"][1] == out["staged"][1]
