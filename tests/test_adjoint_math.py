"""The hand-written VJP / Jacobian kernels of the nonlinear residual, checked
on the CPU with the oracle: VJP = J^T lambda (J assembled from the Jacobian
kernel into an oracle Mat) and both agree with central finite differences
(h = 1e-6) of lambda . F."""
import numpy as np
import pytest

from pyop2_gb300 import workloads as W


def _setup(op2, n=4):
    p = W.build_nonlinear(op2, n=n, seed=2)
    V, C = p["verts"].size, p["cells"].size
    u = op2.Dat(p["verts"], p["u"])
    kappa = op2.Dat(p["cells"], p["kappa"])
    return p, V, C, u, kappa


def residual(op2, p, u_vals, k_vals):
    V = p["verts"].size
    F = op2.Dat(p["verts"], np.zeros(V))
    u = op2.Dat(p["verts"], u_vals)
    k = op2.Dat(p["cells"], k_vals)
    op2.par_loop(op2.Kernel(W.NL_RESIDUAL, "nl_residual"), p["cells"], F(op2.INC, p["c2v"]),
                 p["X"](op2.READ, p["c2v"]), u(op2.READ, p["c2v"]), k(op2.READ))
    return F.data.copy()


def vjp(op2, p, u_vals, k_vals, lam_vals):
    V, C = p["verts"].size, p["cells"].size
    lam = op2.Dat(p["verts"], lam_vals)
    u = op2.Dat(p["verts"], u_vals)
    k = op2.Dat(p["cells"], k_vals)
    du = op2.Dat(p["verts"], np.zeros(V))
    dk = op2.Dat(p["cells"], np.zeros(C))
    op2.par_loop(op2.Kernel(W.NL_RESIDUAL_VJP, "nl_residual_vjp"), p["cells"],
                 lam(op2.READ, p["c2v"]), p["X"](op2.READ, p["c2v"]), u(op2.READ, p["c2v"]),
                 k(op2.READ), du(op2.INC, p["c2v"]), dk(op2.WRITE))
    return du.data.copy(), dk.data.copy()


def jacobian(op2, p, u_vals, k_vals):
    u = op2.Dat(p["verts"], u_vals)
    k = op2.Dat(p["cells"], k_vals)
    sp = op2.Sparsity((p["verts"] ** 1, p["verts"] ** 1), [(p["c2v"], p["c2v"], None)])
    A = op2.Mat(sp)
    op2.par_loop(op2.Kernel(W.NL_RESIDUAL_JACOBIAN, "nl_residual_jac"), p["cells"],
                 A(op2.INC, (p["c2v"], p["c2v"])), p["X"](op2.READ, p["c2v"]),
                 u(op2.READ, p["c2v"]), k(op2.READ))
    A.assemble()
    return A.to_scipy()


def test_vjp_is_jacobian_transpose_and_matches_fd(oracle_op2):
    op2 = oracle_op2
    p = W.build_nonlinear(op2, n=4, seed=2)
    u0, k0, lam = p["u"], p["kappa"], p["lam"]
    du, dk = vjp(op2, p, u0, k0, lam)
    J = jacobian(op2, p, u0, k0)
    jtl = J.T @ lam
    assert np.max(np.abs(du - jtl)) <= 1e-12 * np.max(np.abs(jtl))
    rng = np.random.default_rng(11)
    h = 1e-6
    for _ in range(3):
        d = rng.uniform(-1, 1, len(u0))
        fd = (lam @ residual(op2, p, u0 + h * d, k0) - lam @ residual(op2, p, u0 - h * d, k0)) / (2 * h)
        assert abs(fd - du @ d) <= 1e-6 * max(abs(fd), 1e-3)
        dkk = rng.uniform(-1, 1, len(k0))
        fd = (lam @ residual(op2, p, u0, k0 + h * dkk) - lam @ residual(op2, p, u0, k0 - h * dkk)) / (2 * h)
        assert abs(fd - dk @ dkk) <= 1e-6 * max(abs(fd), 1e-3)


def test_fused_kernel_equals_separate(oracle_op2):
    op2 = oracle_op2
    p = W.build_nonlinear(op2, n=3, seed=4)
    V, C = p["verts"].size, p["cells"].size
    F = op2.Dat(p["verts"], np.zeros(V))
    lam = op2.Dat(p["verts"], p["lam"])
    u = op2.Dat(p["verts"], p["u"])
    k = op2.Dat(p["cells"], p["kappa"])
    du = op2.Dat(p["verts"], np.zeros(V))
    dk = op2.Dat(p["cells"], np.zeros(C))
    op2.par_loop(op2.Kernel(W.NL_RESIDUAL_FUSED, "nl_residual_fused"), p["cells"],
                 F(op2.INC, p["c2v"]), lam(op2.READ, p["c2v"]), p["X"](op2.READ, p["c2v"]),
                 u(op2.READ, p["c2v"]), k(op2.READ), du(op2.INC, p["c2v"]), dk(op2.WRITE))
    F_ref = residual(op2, p, p["u"], p["kappa"])
    du_ref, dk_ref = vjp(op2, p, p["u"], p["kappa"], p["lam"])
    np.testing.assert_allclose(F.data, F_ref, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(du.data, du_ref, rtol=1e-12, atol=1e-14)
    np.testing.assert_allclose(dk.data, dk_ref, rtol=1e-12, atol=1e-14)
