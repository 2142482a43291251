"""Batched persistent launch (configuration 3 shape): many P2 meshes of
uneven size in one launch and in a CUDA graph, against per-mesh launches and
the oracle."""
import numpy as np
import pytest

from pyop2_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_p2_kernel_matches_oracle(gpu_op2, oracle_op2):
    for n in (1, 7):
        g = W.build_p2_batch(gpu_op2, [n], seed=4)[0]
        o = W.build_p2_batch(oracle_op2, [n], seed=4)[0]
        gpu_op2.par_loop(g["kernel"], g["cells"], *g["args"])
        oracle_op2.par_loop(o["kernel"], o["cells"], *o["args"])
        assert rel(g["y"].data_ro, o["y"].data) <= 1e-12
        assert abs(g["g"].data_ro[0] - o["g"].data[0]) <= 1e-12 * abs(o["g"].data[0])


@pytest.mark.parametrize("scatter", ["atomic", "warp", "shared"])
@pytest.mark.parametrize("chunk", [64, 2048])
def test_batched_equals_plain(gpu_op2, chunk, scatter):
    from pyop2_gb300 import _lib
    from pyop2_gb300.batch import BatchedParLoop
    sc = {"atomic": _lib.SCATTER_ATOMIC, "warp": _lib.SCATTER_WARP,
          "shared": _lib.SCATTER_SHARED}[scatter]
    op2 = gpu_op2
    sizes = [1, 3, 9, 17, 40, 5, 64, 2, 23, 31, 12, 50]
    plain = W.build_p2_batch(op2, sizes, seed=9)
    batch = W.build_p2_batch(op2, sizes, seed=9)
    for p in plain:
        op2.par_loop(p["kernel"], p["cells"], *p["args"])
    loops = [op2.ParLoop(p["kernel"], p["cells"], *p["args"]) for p in batch]
    b = BatchedParLoop(loops, chunk=chunk, scatter=sc)
    b.compute()
    for p, q in zip(plain, batch):
        assert rel(q["y"].data_ro, p["y"].data_ro) <= 1e-12
        assert abs(q["g"].data_ro[0] - p["g"].data_ro[0]) <= 1e-12 * abs(p["g"].data_ro[0])
    # graph replay = a second application: everything doubles
    b.capture()
    b.replay()
    for p, q in zip(plain, batch):
        assert rel(q["y"].data_ro, 2 * p["y"].data_ro) <= 1e-12
        assert abs(q["g"].data_ro[0] - 2 * p["g"].data_ro[0]) <= 1e-12 * abs(p["g"].data_ro[0])


def test_batch_rejects_mixed_signatures(gpu_op2):
    from pyop2_gb300.batch import BatchedParLoop
    op2 = gpu_op2
    a = W.build_p2_batch(op2, [3], seed=1)[0]
    s = op2.Set(4)
    d = op2.Dat(s)
    other = op2.ParLoop(op2.Kernel("static void k(double *x) { *x = 1.0; }", "k"), s, d(op2.WRITE))
    with pytest.raises(ValueError):
        BatchedParLoop([op2.ParLoop(a["kernel"], a["cells"], *a["args"]), other])


def test_autotuned_batch_is_correct(gpu_op2):
    """The batch autotuner restores every written argument after its trials,
    and the batch it returns computes what per-mesh launches compute."""
    from pyop2_gb300.batch import autotune_batch
    op2 = gpu_op2
    sizes = [2, 11, 30, 7, 19]
    plain = W.build_p2_batch(op2, sizes, seed=13)
    batch = W.build_p2_batch(op2, sizes, seed=13)
    for p in plain:
        op2.par_loop(p["kernel"], p["cells"], *p["args"])
    loops = [op2.ParLoop(p["kernel"], p["cells"], *p["args"]) for p in batch]
    b, tuned = autotune_batch(loops, chunks=(64, 512), block_sizes=(128,), reps=1)
    assert tuned["scatter"] in ("atomic", "warp", "shared")
    for q in batch:
        assert not np.any(q["y"].data_ro)          # trials left no trace
    b.replay()
    for p, q in zip(plain, batch):
        assert rel(q["y"].data_ro, p["y"].data_ro) <= 1e-12
        assert abs(q["g"].data_ro[0] - p["g"].data_ro[0]) <= 1e-12 * abs(p["g"].data_ro[0])
