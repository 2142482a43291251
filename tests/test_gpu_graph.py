"""LoopGraph: par_loops recorded once into a CUDA graph and replayed.  A
replay must do what calling the loops does, under every INC strategy
(coloured loops record one launch per colour), see host-side changes to
the loops' Dats, and accumulate correctly over repeated replays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STRATEGIES = ["atomic", "warp", "colour", "shared", "staged"]


def _problem(op2, seed):
    from pyop2_gb300 import workloads as W
    p = W.build_p1_3d(op2, n=10, permute=True, seed=seed)
    p["loop"] = op2.ParLoop(p["kernel"], p["cells"], p["y"](op2.INC, p["c2v"]),
                            p["X"](op2.READ, p["c2v"]), p["x"](op2.READ, p["c2v"]))
    area = op2.Global(1, 0.0)
    vol = op2.ParLoop(op2.Kernel("""
static void vol(double *v, const double *X) {
  double a[3], b[3], c[3];
  for (int i = 0; i < 3; ++i) { a[i] = X[3 + i] - X[i]; b[i] = X[6 + i] - X[i];
                                c[i] = X[9 + i] - X[i]; }
  const double d = a[0] * (b[1] * c[2] - b[2] * c[1]) - a[1] * (b[0] * c[2] - b[2] * c[0])
                 + a[2] * (b[0] * c[1] - b[1] * c[0]);
  v[0] += (d < 0 ? -d : d) / 6.0;
}""", "vol"), p["cells"], area(op2.INC), p["X"](op2.READ, p["c2v"]))
    return p, vol, area


@pytest.mark.parametrize("strategy", STRATEGIES)
def test_replay_equals_calls(gpu_op2, strategy):
    from pyop2_gb300.configuration import configuration
    from pyop2_gb300.graph import LoopGraph
    op2 = gpu_op2
    old = configuration["scatter"]
    configuration["scatter"] = strategy
    try:
        p, vol, area = _problem(op2, 3)
        q, vol2, area2 = _problem(op2, 3)
        g = LoopGraph([p["loop"], vol])
        for _ in range(3):
            g.replay()
            q["loop"].compute()
            vol2.compute()
        a, b = p["y"].data_ro, q["y"].data_ro
        assert np.max(np.abs(a - b)) <= 1e-12 * np.max(np.abs(b))
        assert abs(area.data_ro[0] - 3.0) <= 1e-12 and abs(area2.data_ro[0] - 3.0) <= 1e-12
        # host-side changes are uploaded before a replay
        p["x"].data[:] = 0.0
        p["y"].data[:] = 0.0
        g.replay()
        assert np.all(p["y"].data_ro == 0.0)
    finally:
        configuration["scatter"] = old


def test_graph_of_a_batch_and_a_loop(gpu_op2):
    """A BatchedParLoop and a plain loop in one graph."""
    from pyop2_gb300.batch import BatchedParLoop
    from pyop2_gb300.graph import LoopGraph
    op2 = gpu_op2
    ps = [_problem(op2, s) for s in (1, 2)]
    qs = [_problem(op2, s) for s in (1, 2)]
    b = BatchedParLoop([ps[0][0]["loop"], ps[1][0]["loop"]])
    g = LoopGraph([b, ps[0][1]])
    g.replay()
    g.replay()
    for q in qs:
        q[0]["loop"].compute()
        q[0]["loop"].compute()
    qs[0][1].compute()
    qs[0][1].compute()
    for (p, _, _), (q, _, _) in zip(ps, qs):
        a, c = p["y"].data_ro, q["y"].data_ro
        assert np.max(np.abs(a - c)) <= 1e-12 * np.max(np.abs(c))
    assert abs(ps[0][2].data_ro[0] - qs[0][2].data_ro[0]) <= 1e-12
