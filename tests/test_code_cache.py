"""Which par_loops share a compiled wrapper (test/unit/test_caching.py:298-489
semantics), checked on the CPU through the signature key and NVRTC."""
import numpy as np
import pytest

from pyop2_gb300 import op2
from pyop2_gb300.parloop import LegacyParloop

N = 10


@pytest.fixture
def env():
    iterset = op2.Set(N, "iterset")
    indset = op2.Set(N, "indset")
    m1 = op2.Map(iterset, indset, 1, np.arange(N)[::-1])
    m2 = op2.Map(iterset, indset, 2, np.stack([np.arange(N), np.arange(N)[::-1]], 1))
    x = op2.Dat(indset, np.arange(N), np.uint32)
    y = op2.Dat(indset, np.arange(N), np.uint32)
    x2 = op2.Dat(indset ** 2, np.zeros((N, 2)), np.uint32)
    a = op2.Dat(iterset, np.arange(N), np.uint32)
    b = op2.Dat(iterset, np.arange(N), np.uint32)
    return iterset, m1, m2, x, y, x2, a, b


CPY = "static void cpy(unsigned int* dst, unsigned int* src) { *dst = *src; }"
SWAP = """static void swap(unsigned int* x, unsigned int* y)
{ unsigned int t; t = *x; *x = *y; *y = t; }"""


def key(kernel, iterset, *args):
    return LegacyParloop(kernel, iterset, *args).cache_key()


def test_same_args_same_wrapper(env):
    it, m1, m2, x, y, x2, a, b = env
    k = op2.Kernel(CPY, "cpy")
    assert key(k, it, a(op2.WRITE), x(op2.READ, m1)) == \
        key(op2.Kernel(CPY, "cpy"), it, a(op2.WRITE), x(op2.READ, m1))


def test_different_kernel_text(env):
    it, m1, m2, x, y, x2, a, b = env
    k1 = op2.Kernel(CPY, "cpy")
    k2 = op2.Kernel(CPY.replace("dst", "DST").replace("src", "SRC"), "cpy")
    assert key(k1, it, a(op2.WRITE), x(op2.READ, m1)) != key(k2, it, a(op2.WRITE), x(op2.READ, m1))


def test_swapped_args_of_same_shape_share(env):
    it, m1, m2, x, y, x2, a, b = env
    k = op2.Kernel(SWAP, "swap")
    assert key(k, it, x(op2.RW, m1), y(op2.RW, m1)) == key(k, it, y(op2.RW, m1), x(op2.RW, m1))
    assert key(k, it, a(op2.RW), b(op2.RW)) == key(k, it, b(op2.RW), a(op2.RW))


def test_map_identity_matters(env):
    """Two args through one map differ from two args through two maps."""
    it, m1, m2, x, y, x2, a, b = env
    m1b = op2.Map(it, m1.toset, 1, np.arange(N))
    k = op2.Kernel(SWAP, "swap")
    assert key(k, it, x(op2.RW, m1), y(op2.RW, m1)) != key(k, it, x(op2.RW, m1), y(op2.RW, m1b))


def test_dtype_dim_and_access_matter(env):
    it, m1, m2, x, y, x2, a, b = env
    k = op2.Kernel("static void k(void *x) {}", "k")
    d32 = op2.Dat(it, np.arange(N), np.int32)
    assert key(k, it, a(op2.WRITE)) != key(k, it, d32(op2.WRITE))
    gu = op2.Global(1, 0, np.uint32)
    gd = op2.Global(1, 0, np.float64)
    assert key(k, it, gu(op2.INC)) != key(k, it, gd(op2.INC))
    assert key(k, it, x(op2.READ, m1)) != key(k, it, x2(op2.READ, m1))
    assert key(k, it, x(op2.READ, m1)) != key(k, it, x(op2.INC, m1))
    assert key(k, it, x2(op2.INC, m2)) == key(k, it, x2(op2.INC, m2))


def test_void_pointer_kernel_compiles(env):
    """Kernels declaring void* arguments compile (the reference passes every
    argument as void* through ctypes)."""
    from pyop2_gb300.csrc import build
    build.build()
    from pyop2_gb300.parloop import compile_signature
    it, m1, m2, x, y, x2, a, b = env
    pl = LegacyParloop(op2.Kernel("static void k(void *x) {}", "k"), it, x2(op2.INC, m2))
    t, args = pl._signature()
    c = compile_signature(pl.local_kernel.source, "k", pl._loop_desc(0, 256), args, t.key(),
                          arch="sm_103a")
    assert c.nptrs == 2
