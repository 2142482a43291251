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


# ---- test/unit/test_linalg.py, case by case
NEL = 8


@pytest.fixture
def xy(gpu_op2):
    op2 = gpu_op2
    dset = op2.DataSet(op2.Set(NEL), 1)
    x = op2.Dat(dset, None, np.float64, "x")
    y = op2.Dat(dset, np.arange(1, NEL + 1), np.float64, "y")
    yi = op2.Dat(dset, np.arange(1, NEL + 1), np.int64, "y")
    return op2, x, y, yi


@pytest.fixture
def xy2(gpu_op2):
    op2 = gpu_op2
    x2 = op2.Dat(op2.Set(NEL, "s1") ** (1, 2), np.zeros(2 * NEL), np.float64, "x")
    y2 = op2.Dat(op2.Set(NEL, "s2") ** (2, 1), np.zeros(2 * NEL), np.float64, "y")
    return x2, y2


def test_linalg_op(xy):
    op2, x, y, yi = xy
    x._data = 2 * y.data
    assert all((x + y).data == 3 * y.data)
    assert all((x - y).data == y.data)
    assert all((x * y).data == 2 * y.data * y.data)
    assert all((x / y).data == 2.0)
    x._data = y.data + 1.0
    assert all(x.data == (y + 1.0).data) and all(x.data == (1.0 + y).data)
    x._data = y.data - 1.0
    assert all(x.data == (y - 1.0).data)
    x._data = 1.0 - y.data
    assert all(x.data == (1.0 - y).data)
    x._data = 2 * y.data
    assert all(x.data == (y * 2.0).data) and all(x.data == (2.0 * y).data)
    assert all((x / 2.0).data == y.data)


def test_linalg_pos_neg_copy(xy):
    op2, x, y, yi = xy
    z = +y
    assert all(z.data == y.data) and z is not y
    z = -y
    assert all(z.data == -y.data) and z is not y


@pytest.mark.parametrize("op", ["+", "-", "*", "/"])
def test_linalg_result_dtype_is_left_operand(xy, op):
    op2, x, y, yi = xy
    f = {"+": lambda a, b: a + b, "-": lambda a, b: a - b, "*": lambda a, b: a * b,
         "/": lambda a, b: a / b}[op]
    assert f(y, yi).data.dtype == np.float64
    assert f(yi, y).data.dtype == np.int64


@pytest.mark.parametrize("op", ["+", "-", "*", "/"])
def test_linalg_shape_mismatch(xy2, op):
    x2, y2 = xy2
    f = {"+": lambda a, b: a + b, "-": lambda a, b: a - b, "*": lambda a, b: a * b,
         "/": lambda a, b: a / b}[op]
    with pytest.raises(ValueError):
        f(x2, y2)


@pytest.mark.parametrize("op", ["+=", "-=", "*=", "/="])
def test_linalg_iop_shape_mismatch(xy2, op):
    x2, y2 = xy2
    with pytest.raises(ValueError):
        if op == "+=":
            x2 += y2
        elif op == "-=":
            x2 -= y2
        elif op == "*=":
            x2 *= y2
        else:
            x2 /= y2


def test_linalg_and_parloop(xy):
    op2, x, y, yi = xy
    x._data = np.zeros(x.dataset.total_size, dtype=np.float64)
    op2.par_loop(op2.Kernel('static void k(double *x) { *x = 1.0; }', 'k'), x.dataset.set,
                 x(op2.WRITE))
    assert all((x + y).data == y.data + 1)


def test_linalg_iop(xy):
    op2, x, y, yi = xy
    x._data = 2 * y.data
    x += y
    assert all(x.data == 3 * y.data)
    x._data = 2 * y.data
    x -= y
    assert all(x.data == y.data)
    x._data = 2 * y.data
    x *= y
    assert all(x.data == 2 * y.data * y.data)
    x._data = 2 * y.data
    x /= y
    assert all(x.data == 2.0)
    x._data = 2 * y.data
    x /= 2.0
    assert all(x.data == y.data)


def test_linalg_iop_scalar(xy):
    op2, x, y, yi = xy
    x._data = y.data + 1.0
    y += 1.0
    assert all(x.data == y.data)
    x._data = y.data - 1.0
    y -= 1.0
    assert all(x.data == y.data)
    x._data = 2 * y.data
    y *= 2.0
    assert all(x.data == y.data)


@pytest.mark.parametrize("op", ["+=", "-=", "*=", "/="])
def test_linalg_iop_dtype(xy, op):
    op2, x, y, yi = xy
    for a, b, dt in ((y, yi, np.float64), (yi, y, np.int64)):
        if op == "+=":
            a += b
        elif op == "-=":
            a -= b
        elif op == "*=":
            a *= b
        else:
            a /= b
        assert a.data.dtype == dt


def test_linalg_scalar(gpu_op2):
    op2 = gpu_op2
    s = op2.Set(2)
    n = op2.Dat(s, [3, 4], np.float64, "n")
    assert abs(n.norm - 5) < 1e-12
    o = op2.Dat(s, [4, 5], np.float64)
    assert abs(n.inner(o) - 32) < 1e-12 and abs(o.inner(n) - 32) < 1e-12
