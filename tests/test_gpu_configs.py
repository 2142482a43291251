"""Benchmark configurations on the GPU against the oracle (small sizes) and
through size-independent properties (full sizes)."""
import numpy as np
import pytest

from pyop2_gb300 import workloads
from pyop2_gb300 import workloads as W

pytestmark = pytest.mark.gpu

STRATEGIES = ["atomic", "warp", "colour", "shared", "staged", "atomic_cells2"]


@pytest.fixture(params=STRATEGIES)
def strategy(request, gpu_op2):
    from pyop2_gb300.configuration import configuration
    old = configuration["scatter"], configuration["cells_per_thread"]
    # "atomic_cells2": hardware atomics, two cells per thread per sweep step
    configuration["scatter"] = request.param.split("_")[0]
    configuration["cells_per_thread"] = 2 if request.param.endswith("cells2") else 1
    yield request.param
    configuration["scatter"], configuration["cells_per_thread"] = old


def relerr(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_config1_p1_2d(gpu_op2, oracle_op2, strategy):
    g = workloads.build_p1_2d(gpu_op2, n=64, seed=0)
    o = workloads.build_p1_2d(oracle_op2, n=64, seed=0)
    g["run"]()
    o["run"]()
    assert abs(g["area"].data[0] - 1.0) < 1e-12
    assert abs(g["area"].data[0] - o["area"].data[0]) < 1e-14
    assert relerr(g["y"].data_ro, o["y"].data) <= 1e-12


@pytest.mark.parametrize("permute", [False, True])
def test_config2a_small_vs_oracle(gpu_op2, oracle_op2, strategy, permute):
    g = workloads.build_p1_3d(gpu_op2, n=24, permute=permute, seed=3)
    o = workloads.build_p1_3d(oracle_op2, n=24, permute=permute, seed=3)
    g["run"]()
    o["run"]()
    assert relerr(g["y"].data_ro, o["y"].data) <= 1e-12


@pytest.mark.parametrize("permute", [False, True])
def test_config2a_full_size_properties(gpu_op2, permute):
    """128^3 x 6 tets: the Laplacian annihilates constants (sum y = 0 up to
    rounding) and the action is linear."""
    op2 = gpu_op2
    p = workloads.build_p1_3d(op2, n=128, permute=permute, seed=0)
    x0 = p["x"].data_ro.copy()
    p["run"]()
    y1 = p["y"].data_ro.copy()
    scale = np.abs(y1).max()
    assert abs(y1.sum()) <= 1e-9 * scale * np.sqrt(len(y1))
    # linearity: A(2x) = 2 A(x)
    p["x"].data[:] = 2 * x0
    p["y"].zero()
    p["run"]()
    assert relerr(p["y"].data_ro, 2 * y1) <= 1e-12
    # constant field -> zero action
    p["x"].data[:] = 1.0
    p["y"].zero()
    p["run"]()
    assert np.abs(p["y"].data_ro).max() <= 1e-12 * scale


@pytest.mark.parametrize("permute", [False, True])
def test_full_size_colouring_is_valid(gpu_op2, permute):
    """Jones-Plassmann colouring of the 12.58 M tets: no two cells of one colour
    share a vertex; every cell appears exactly once."""
    import torch
    from pyop2_gb300.parloop import colour_plan
    op2 = gpu_op2
    p = W.build_p1_3d(op2, n=128, permute=permute, seed=0)
    lp = op2.ParLoop(p["kernel"], p["cells"], p["y"](op2.INC, p["c2v"]),
                     p["X"](op2.READ, p["c2v"]), p["x"](op2.READ, p["c2v"]))
    plan = colour_plan(lp)
    assert plan is not None and 8 <= plan.ncolours <= 256
    assert plan.ptr[-1] == p["cells"].size
    order = plan.order[:p["cells"].size].long()
    assert torch.unique(order).numel() == p["cells"].size
    assert plan.validate([p["c2v"]])
