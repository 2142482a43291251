"""The benchmark configurations at their benchmarked sizes, on the GPU,
against the oracle on the same seeded inputs.

- 2a: the P1 tet action on 128^3 x 6 = 12,582,912 cells, lexicographic and
  randomly permuted vertex numbering: y within 1e-12 relative.
- 2b: the sparsity of the same mesh (31,802,497 nonzeros), row pointers and
  column indices bit for bit, both numberings; the assembled CSR values of
  the 4x4 element matrices within 1e-12.
- 3: the 256 P2 meshes of the batch (seed 0, 46.4 M cells) run as one
  batched launch replayed from its CUDA graph: every mesh's y and Global.
- 4: the nonlinear residual on 64^3 x 6 tets through torch.autograd
  (AdjointParLoop): F, dL/du and dL/dkappa against the oracle's residual and
  VJP loops.

The reference semantics restated by the oracle: pyop2/codegen/builder.py:
303-410 (Dat pack/unpack), 501-606 (Mat insertion) and pyop2/sparsity.pyx:
178-405 (the pattern).  The extruded prism configuration (5) is in
test_gpu_full_size_prisms.py.
"""
import numpy as np
import pytest

from pyop2_gb300 import workloads as W
from test_adjoint_math import residual, vjp

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.fixture(scope="module")
def c2a_oracle(oracle_op2):
    out = {}
    for permute in (False, True):
        o = W.build_p1_3d(oracle_op2, n=128, permute=permute, seed=0)
        o["run"]()
        out[permute] = o["y"].data.copy()
    return out


@pytest.mark.parametrize("scatter", ["atomic", "staged"])
@pytest.mark.parametrize("permute", [False, True])
def test_config2a_full_size_vs_oracle(gpu_op2, c2a_oracle, permute, scatter):
    from pyop2_gb300.configuration import configuration
    g = W.build_p1_3d(gpu_op2, n=128, permute=permute, seed=0)
    assert g["cells"].size == 12582912 and g["verts"].size == 2146689
    old = configuration["scatter"]
    configuration["scatter"] = scatter
    try:
        g["run"]()
    finally:
        configuration["scatter"] = old
    assert rel(g["y"].data_ro, c2a_oracle[permute]) <= 1e-12


def _pattern(op2, p):
    return op2.Sparsity((p["verts"] ** 1, p["verts"] ** 1), [(p["c2v"], p["c2v"], None)])


@pytest.mark.parametrize("permute", [False, True])
def test_config2b_full_size_pattern_and_values_vs_oracle(gpu_op2, oracle_op2, permute):
    g = W.build_p1_3d(gpu_op2, n=128, permute=permute, seed=0)
    o = W.build_p1_3d(oracle_op2, n=128, permute=permute, seed=0)
    sp, spo = _pattern(gpu_op2, g), _pattern(oracle_op2, o)
    rp, ci = sp.csr()
    assert len(spo.colidx) == 31802497
    assert np.array_equal(rp, spo.rowptr)
    assert np.array_equal(ci, spo.colidx)
    assert np.array_equal(sp.nnz, spo.nnz)
    A, Ao = gpu_op2.Mat(sp), oracle_op2.Mat(spo)
    k = W.P1_3D_LAPLACE_MATRIX
    gpu_op2.par_loop(gpu_op2.Kernel(k, "p1_laplace_3d_mat"), g["cells"],
                     A(gpu_op2.INC, (g["c2v"], g["c2v"])), g["X"](gpu_op2.READ, g["c2v"]))
    oracle_op2.par_loop(oracle_op2.Kernel(k, "p1_laplace_3d_mat"), o["cells"],
                        Ao(oracle_op2.INC, (o["c2v"], o["c2v"])), o["X"](oracle_op2.READ, o["c2v"]))
    A.assemble()
    v = A.csr()[2].reshape(-1)
    vo = Ao.values_bcsr.reshape(-1)
    assert np.max(np.abs(v - vo)) <= 1e-12 * np.max(np.abs(vo))


def test_config3_all_256_meshes_batched_graph_vs_oracle(gpu_op2, oracle_op2):
    """The batch exactly as the benchmark builds it, tuned by the batch
    autotuner (which restores every written argument after its trials), then
    one replay of the tuned graph."""
    from pyop2_gb300 import meshes
    from pyop2_gb300.batch import autotune_batch
    sizes = meshes.batch_sizes(256, seed=0)
    gp = W.build_p2_batch(gpu_op2, sizes, seed=0)
    loops = [gpu_op2.ParLoop(p["kernel"], p["cells"], *p["args"]) for p in gp]
    assert sum(lp.iterset.size for lp in loops) == 46425882
    batch, tuned = autotune_batch(loops, reps=1)
    batch.replay()
    op = W.build_p2_batch(oracle_op2, sizes, seed=0)
    worst_y = worst_g = 0.0
    for i, (p, q) in enumerate(zip(gp, op)):
        oracle_op2.par_loop(q["kernel"], q["cells"], *q["args"])
        worst_y = max(worst_y, rel(p["y"].data_ro, q["y"].data))
        gq = q["g"].data[0]
        worst_g = max(worst_g, abs(p["g"].data_ro[0] - gq) / abs(gq))
    assert worst_y <= 1e-12, (worst_y, tuned)
    assert worst_g <= 1e-12, (worst_g, tuned)


def test_config4_full_size_autograd_vs_oracle(gpu_op2, oracle_op2):
    """64^3 x 6 = 1,572,864 tets: the residual and the gradients of
    lambda . F that torch.autograd returns through AdjointParLoop."""
    import torch
    from test_gpu_adjoint import make_loop
    g = W.build_nonlinear(gpu_op2, n=64, seed=0)
    o = W.build_nonlinear(oracle_op2, n=64, seed=0)
    assert g["cells"].size == 1572864
    loop = make_loop(gpu_op2, g)
    dev = torch.device("cuda")
    u = torch.tensor(g["u"], device=dev, requires_grad=True)
    k = torch.tensor(g["kappa"], device=dev, requires_grad=True)
    lam = torch.tensor(g["lam"], device=dev)
    F = loop(u, k)
    (lam * F).sum().backward()
    F_ref = residual(oracle_op2, o, o["u"], o["kappa"])
    du_ref, dk_ref = vjp(oracle_op2, o, o["u"], o["kappa"], o["lam"])
    assert rel(F.detach().cpu().numpy(), F_ref) <= 1e-12
    assert rel(u.grad.cpu().numpy(), du_ref) <= 1e-12
    assert rel(k.grad.cpu().numpy(), dk_ref) <= 1e-12
