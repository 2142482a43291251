"""Prism elasticity kernels checked on the CPU with the oracle: the
assembled BAIJ matrix is symmetric and reproduces the matrix-free action for
every right-hand side; the VJP equals K w and central differences in the
Lame fields; rigid motions are in the kernel of the operator."""
import numpy as np

from pyop2_gb300 import workloads as W

NR = W.PRISM_NRHS


def setup(op2, n=3, layers=4, seed=1):
    return W.build_prisms(op2, n=n, layers=layers, seed=seed)


def action(op2, p, u_vals, lame_vals):
    nodes = p["nodes"]
    y = op2.Dat(op2.DataSet(nodes, (NR, 3)), np.zeros((p["nnodes"], NR, 3)))
    u = op2.Dat(op2.DataSet(nodes, (NR, 3)), u_vals)
    L = op2.Dat(op2.DataSet(p["prisms"], 2), lame_vals)
    op2.par_loop(op2.Kernel(W.PRISM_ELASTICITY_ACTION, "prism_elasticity"), p["cells"],
                 y(op2.INC, p["c2n"]), p["X"](op2.READ, p["c2n"]), u(op2.READ, p["c2n"]),
                 L(op2.READ, p["c2c"]))
    return y.data.copy()


def vjp(op2, p, w_vals, u_vals, lame_vals):
    nodes = p["nodes"]
    w = op2.Dat(op2.DataSet(nodes, (NR, 3)), w_vals)
    u = op2.Dat(op2.DataSet(nodes, (NR, 3)), u_vals)
    L = op2.Dat(op2.DataSet(p["prisms"], 2), lame_vals)
    du = op2.Dat(op2.DataSet(nodes, (NR, 3)), np.zeros((p["nnodes"], NR, 3)))
    dL = op2.Dat(op2.DataSet(p["prisms"], 2), np.zeros((p["ncell"], 2)))
    op2.par_loop(op2.Kernel(W.PRISM_ELASTICITY_VJP, "prism_elasticity_vjp"), p["cells"],
                 w(op2.READ, p["c2n"]), p["X"](op2.READ, p["c2n"]), u(op2.READ, p["c2n"]),
                 L(op2.READ, p["c2c"]), du(op2.INC, p["c2n"]), dL(op2.WRITE, p["c2c"]))
    return du.data.copy(), dL.data.copy()


def matrix(op2, p, lame_vals):
    nodes = p["nodes"]
    sp = op2.Sparsity((nodes ** 3, nodes ** 3), [(p["c2n"], p["c2n"], None)])
    A = op2.Mat(sp)
    L = op2.Dat(op2.DataSet(p["prisms"], 2), lame_vals)
    op2.par_loop(op2.Kernel(W.PRISM_ELASTICITY_MATRIX, "prism_elasticity_mat"), p["cells"],
                 A(op2.INC, (p["c2n"], p["c2n"])), p["X"](op2.READ, p["c2n"]),
                 L(op2.READ, p["c2c"]))
    A.assemble()
    return A.to_scipy()


def test_matrix_symmetric_and_equals_action(oracle_op2):
    op2 = oracle_op2
    p = setup(op2)
    lame = op2_lame(p)
    A = matrix(op2, p, lame)
    Ad = A.toarray()
    assert np.max(np.abs(Ad - Ad.T)) <= 1e-13 * np.max(np.abs(Ad))
    y = action(op2, p, p["u"], lame)
    for r in range(NR):
        ref = A @ p["u"][:, r, :].reshape(-1)
        assert np.max(np.abs(y[:, r, :].reshape(-1) - ref)) <= 1e-12 * np.max(np.abs(ref))


def op2_lame(p):
    rng = np.random.default_rng(3)
    return np.stack([rng.lognormal(0, 0.3, p["ncell"]), rng.lognormal(0, 0.3, p["ncell"])], axis=1)


def test_rigid_motions_are_free(oracle_op2):
    op2 = oracle_op2
    p = setup(op2)
    lame = op2_lame(p)
    nc = p["X"].data.reshape(-1, 3)
    u = np.zeros((p["nnodes"], NR, 3))
    u[:, 0, 0] = 1.0                       # translation
    u[:, 1, 0], u[:, 1, 1] = -nc[:, 1], nc[:, 0]   # rotation about z
    y = action(op2, p, u, lame)
    assert np.max(np.abs(y[:, :2, :])) <= 1e-12


def test_vjp(oracle_op2):
    op2 = oracle_op2
    p = setup(op2)
    lame = op2_lame(p)
    du, dL = vjp(op2, p, p["w"], p["u"], lame)
    # dL/du = K w
    Kw = action(op2, p, p["w"], lame)
    assert np.max(np.abs(du - Kw)) <= 1e-12 * np.max(np.abs(Kw))
    # Lame gradients by central differences of w . K(lame) u
    h = 1e-6
    rng = np.random.default_rng(9)
    for comp in (0, 1):
        d = np.zeros_like(lame)
        d[:, comp] = rng.uniform(-1, 1, len(lame))
        fp = np.sum(p["w"] * action(op2, p, p["u"], lame + h * d))
        fm = np.sum(p["w"] * action(op2, p, p["u"], lame - h * d))
        fd = (fp - fm) / (2 * h)
        an = np.sum(dL * d)
        assert abs(fd - an) <= 1e-7 * abs(an)
