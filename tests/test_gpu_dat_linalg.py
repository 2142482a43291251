"""Dat pointwise linear algebra (test/unit/test_linalg.py semantics) run as
generated direct par_loops on the GPU, against numpy."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def dats(gpu_op2):
    op2 = gpu_op2
    s = op2.Set((3, 7, 9))           # ghosts (7..8) are not touched
    rng = np.random.default_rng(1)
    a = op2.Dat(s ** 2, rng.uniform(1, 2, (9, 2)))
    b = op2.Dat(s ** 2, rng.uniform(1, 2, (9, 2)))
    return op2, s, a, b


def test_binary_ops(dats):
    op2, s, a, b = dats
    A, B = a.data_ro.copy(), b.data_ro.copy()
    np.testing.assert_allclose((a + b).data_ro, A + B)
    np.testing.assert_allclose((a - b).data_ro, A - B)
    np.testing.assert_allclose((a * b).data_ro, A * B)
    np.testing.assert_allclose((a / b).data_ro, A / B)
    np.testing.assert_allclose((a * 2.5).data_ro, A * 2.5)
    np.testing.assert_allclose((3.0 - a).data_ro, 3.0 - A)
    np.testing.assert_allclose((-a).data_ro, -A)
    np.testing.assert_allclose((2.0 * a).data_ro, 2.0 * A)


def test_inplace_ops_and_reductions(dats):
    op2, s, a, b = dats
    A, B = a.data_ro.copy(), b.data_ro.copy()
    a += b
    np.testing.assert_allclose(a.data_ro, A + B)
    a -= 1.0
    np.testing.assert_allclose(a.data_ro, A + B - 1)
    a *= a
    np.testing.assert_allclose(a.data_ro, (A + B - 1) ** 2)
    a /= 2.0
    np.testing.assert_allclose(a.data_ro, (A + B - 1) ** 2 / 2)
    assert abs(b.inner(b) - np.sum(B * B)) <= 1e-12 * np.sum(B * B)
    assert abs(b.norm - np.sqrt(np.sum(B * B))) <= 1e-12 * np.sqrt(np.sum(B * B))


def test_shape_mismatch(dats):
    op2, s, a, b = dats
    c = op2.Dat(s ** 3)
    with pytest.raises(ValueError):
        a + c
