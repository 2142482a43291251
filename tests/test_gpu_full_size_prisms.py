"""Configuration 5 at its benchmarked size on the GPU against the oracle:
256^2 x 2 base triangles extruded to 64 layers (8,388,608 prisms, 4,293,185
nodes), P1 displacement with 8 right-hand sides.

- the blocked (3x3 BAIJ) sparsity, 88,835,777 blocks, bit for bit
  (pyop2/sparsity.pyx:305-387 for the extruded pattern);
- the matrix-free 8-RHS action and its adjoint (displacement and Lame
  gradients) within 1e-12 relative (pyop2/codegen/builder.py:81-125 for the
  extruded map offsets).

Kept in a module of its own: the oracle's pattern and prism loops take the
longest of the full-size checks (tens of seconds on one host core).
"""
import numpy as np
import pytest

from pyop2_gb300 import workloads as W
from test_prism_math import action, vjp

pytestmark = pytest.mark.gpu


def rel(a, b):
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


@pytest.fixture(scope="module")
def prisms(gpu_op2, oracle_op2):
    g = W.build_prisms(gpu_op2, n=256, layers=65, seed=0)
    o = W.build_prisms(oracle_op2, n=256, layers=65, seed=0)
    assert g["ncell"] == 8388608 and g["nnodes"] == 4293185
    return g, o


def test_config5_full_size_baij_pattern_vs_oracle(gpu_op2, oracle_op2, prisms):
    g, o = prisms
    sp = gpu_op2.Sparsity((g["nodes"] ** 3, g["nodes"] ** 3), [(g["c2n"], g["c2n"], None)])
    spo = oracle_op2.Sparsity((o["nodes"] ** 3, o["nodes"] ** 3), [(o["c2n"], o["c2n"], None)])
    rp, ci = sp.csr()
    assert len(spo.colidx) == 88835777
    assert np.array_equal(rp, spo.rowptr)
    assert np.array_equal(ci, spo.colidx)
    assert np.array_equal(sp.nnz, spo.nnz)


def test_config5_full_size_action_and_adjoint_vs_oracle(gpu_op2, oracle_op2, prisms):
    g, o = prisms
    lame = o["L"].data_ro
    assert rel(action(gpu_op2, g, g["u"], lame), action(oracle_op2, o, o["u"], lame)) <= 1e-12
    du, dL = vjp(gpu_op2, g, g["w"], g["u"], lame)
    duo, dLo = vjp(oracle_op2, o, o["w"], o["u"], lame)
    assert rel(du, duo) <= 1e-12
    assert rel(dL, dLo) <= 1e-12
