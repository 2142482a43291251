"""Adjoint of the nonlinear residual on the GPU (configuration 4):
torch.autograd through AdjointParLoop against the oracle's VJP, against
J^T lambda with J assembled on the GPU, and against central finite
differences at full size (64^3 x 6 tets)."""
import numpy as np
import pytest

from pyop2_gb300 import workloads as W
from test_adjoint_math import jacobian, residual, vjp

pytestmark = pytest.mark.gpu


def make_loop(op2, p):
    from pyop2_gb300.adjoint import AdjointParLoop
    return AdjointParLoop(
        p["cells"], op2.Kernel(W.NL_RESIDUAL, "nl_residual"),
        op2.Kernel(W.NL_RESIDUAL_VJP, "nl_residual_vjp"),
        output=(p["verts"] ** 1, p["c2v"]),
        inputs=[(p["verts"] ** 1, p["c2v"]), (p["cells"] ** 1, None)],
        constants=[(p["X"], p["c2v"])],
        fused_kernel=op2.Kernel(W.NL_RESIDUAL_FUSED, "nl_residual_fused"))


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_autograd_matches_oracle_vjp_and_jacobian(gpu_op2, oracle_op2):
    import torch
    op2 = gpu_op2
    p = W.build_nonlinear(op2, n=6, seed=3)
    po = W.build_nonlinear(oracle_op2, n=6, seed=3)
    loop = make_loop(op2, p)
    dev = torch.device("cuda")
    u = torch.tensor(p["u"], device=dev, requires_grad=True)
    k = torch.tensor(p["kappa"], device=dev, requires_grad=True)
    lam = torch.tensor(p["lam"], device=dev)
    F = loop(u, k)
    F_ref = residual(oracle_op2, po, po["u"], po["kappa"])
    assert rel(F.detach().cpu().numpy(), F_ref) <= 1e-12
    (lam * F).sum().backward()
    du_ref, dk_ref = vjp(oracle_op2, po, po["u"], po["kappa"], po["lam"])
    assert rel(u.grad.cpu().numpy(), du_ref) <= 1e-12
    assert rel(k.grad.cpu().numpy(), dk_ref) <= 1e-12
    # J^T lambda with J assembled on the GPU
    J = jacobian(op2, p, p["u"], p["kappa"])
    assert rel(u.grad.cpu().numpy(), J.T @ p["lam"]) <= 1e-12
    # fused forward + adjoint
    F2, (du2, dk2) = loop.fused(lam, u.detach(), k.detach())
    assert rel(F2.cpu().numpy(), F_ref) <= 1e-12
    assert rel(du2.cpu().numpy(), du_ref) <= 1e-12
    assert rel(dk2.cpu().numpy(), dk_ref) <= 1e-12


def test_full_size_central_differences(gpu_op2):
    """64^3 x 6 = 1,572,864 cells: directional derivatives of lambda . F by
    central differences (h = 1e-6) match the adjoint gradient."""
    import torch
    op2 = gpu_op2
    p = W.build_nonlinear(op2, n=64, seed=0)
    loop = make_loop(op2, p)
    dev = torch.device("cuda")
    u = torch.tensor(p["u"], device=dev)
    k = torch.tensor(p["kappa"], device=dev)
    lam = torch.tensor(p["lam"], device=dev)
    du, dk = loop.vjp(lam, u, k)
    gen = torch.Generator(device="cpu").manual_seed(5)
    h = 1e-6
    for grad, which in ((du, 0), (dk, 1)):
        d = (torch.rand(grad.shape, generator=gen, dtype=torch.float64) * 2 - 1).to(dev)
        xp = [u, k]
        xm = [u, k]
        xp[which] = xp[which] + h * d
        xm[which] = xm[which] - h * d
        fd = ((lam * loop.forward_values(*xp)).sum() - (lam * loop.forward_values(*xm)).sum()) / (2 * h)
        an = (grad * d).sum()
        assert abs(float(fd - an)) <= 1e-6 * abs(float(an)), (which, float(fd), float(an))
