"""Stored oracle outputs (tests/golden/golden.npz, written by
tests/golden/make_golden.py) on small seeded instances of the benchmark
configurations: the oracle must still produce them (CPU), and so must the
GPU (-m gpu).  Integer arrays (the CSR pattern) are compared exactly, FP64
arrays to 1e-12 relative (compilers on different hosts may contract the
oracle's C differently)."""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402

GOLDEN = dict(np.load(os.path.join(HERE, "golden", "golden.npz")))


def _check(got):
    assert set(got) == set(GOLDEN)
    for k, want in GOLDEN.items():
        g = np.asarray(got[k])
        assert g.shape == want.shape and g.dtype == want.dtype, k
        if np.issubdtype(want.dtype, np.integer):
            assert np.array_equal(g, want), k
        else:
            scale = max(np.max(np.abs(want)), 1e-300)
            assert np.max(np.abs(g - want)) <= 1e-12 * scale, k


def test_oracle_reproduces_fixtures(oracle_op2):
    _check(make_golden.compute(oracle_op2))


@pytest.mark.gpu
def test_gpu_matches_fixtures(gpu_op2):
    _check(make_golden.compute(gpu_op2))
