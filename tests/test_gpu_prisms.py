"""Configuration 5: extruded prism vector elasticity on the GPU, 8 RHS.
Small meshes against the oracle (action, VJP, BAIJ pattern and values); the
full 256^2 x 64 mesh through the exact block count and SpMV = action."""
import numpy as np
import pytest

from pyop2_gb300 import workloads as W
from test_prism_math import action, matrix, op2_lame, vjp

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.max(np.abs(a - b)) / np.max(np.abs(b))


def test_action_and_vjp_vs_oracle(gpu_op2, oracle_op2):
    p = W.build_prisms(gpu_op2, n=8, layers=6, seed=2)
    po = W.build_prisms(oracle_op2, n=8, layers=6, seed=2)
    lame = op2_lame(p)
    assert rel(action(gpu_op2, p, p["u"], lame), action(oracle_op2, po, po["u"], lame)) <= 1e-12
    du, dL = vjp(gpu_op2, p, p["w"], p["u"], lame)
    duo, dLo = vjp(oracle_op2, po, po["w"], po["u"], lame)
    assert rel(du, duo) <= 1e-12
    assert rel(dL, dLo) <= 1e-12


def test_baij_pattern_and_values_vs_oracle(gpu_op2, oracle_op2):
    p = W.build_prisms(gpu_op2, n=6, layers=5, seed=3)
    po = W.build_prisms(oracle_op2, n=6, layers=5, seed=3)
    lame = op2_lame(p)
    A = matrix(gpu_op2, p, lame)
    Ao = matrix(oracle_op2, po, lame)
    assert np.array_equal(A.indptr, Ao.indptr) and np.array_equal(A.indices, Ao.indices)
    assert rel(A.data, Ao.data) <= 1e-12


def test_full_size_baij_and_spmv(gpu_op2):
    op2 = gpu_op2
    p = W.build_prisms(op2, n=256, layers=65, seed=0)
    sp = op2.Sparsity((p["nodes"] ** 3, p["nodes"] ** 3), [(p["c2n"], p["c2n"], None)])
    # base pattern 257^2 + 2 (2*256*257 + 256^2) couplings, each on 65 + 2*64 levels
    assert sp.nblocks == (257 * 257 + 2 * (2 * 256 * 257 + 256 * 256)) * (65 + 2 * 64) == 88835777
    A = op2.Mat(sp)
    op2.par_loop(op2.Kernel(W.PRISM_ELASTICITY_MATRIX, "prism_elasticity_mat"), p["cells"],
                 A(op2.INC, (p["c2n"], p["c2n"])), p["X"](op2.READ, p["c2n"]),
                 p["L"](op2.READ, p["c2c"]))
    A.assemble()
    y = action(op2, p, p["u"], p["L"].data_ro)
    for r in (0, 5):
        x = op2.Dat(p["nodes"] ** 3, p["u"][:, r, :].copy())
        yr = op2.Dat(p["nodes"] ** 3)
        A.mult(x, yr)
        assert rel(yr.data_ro, y[:, r, :]) <= 1e-12
