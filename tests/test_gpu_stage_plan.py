"""Staging plans (op2g_stage_plan_count / _fill) against a numpy restatement
of the local renumbering of the historical OP2 execution plan
(doc/sphinx/source/plan.rst:21-39): per partition of `block` iterations, the
sorted distinct non-negative map values, and per map entry the position of
its value in that list (0xFFFF for a negative entry)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def plan_model(vals, block):
    n, ar = vals.shape
    off, ind, loc = [0], [], np.full(n * ar, 0xFFFF, dtype=np.int64)
    for c0 in range(0, n, block):
        v = vals[c0:c0 + block].reshape(-1)
        u = np.unique(v[v >= 0])
        ind.append(u)
        off.append(off[-1] + len(u))
        pos = np.searchsorted(u, v)
        ok = v >= 0
        loc[c0 * ar:c0 * ar + len(v)][ok] = pos[ok]
    return np.array(off), (np.concatenate(ind) if ind else np.zeros(0, np.int32)), loc


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
    off, ind, loc = plan_model(vals, block)
    assert np.array_equal(p.ind_off.cpu().numpy(), off)
    assert p.total == off[-1]
    assert np.array_equal(p.ind_map.cpu().numpy()[:off[-1]], ind)
    got = p.loc_map.cpu().numpy()[:n * arity].astype(np.int64) & 0xFFFF
    assert np.array_equal(got, loc)
    assert p.max_unique == int(np.max(np.diff(off)))


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
