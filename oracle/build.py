"""oracle/build.py -- TEST INFRASTRUCTURE ONLY.

Compiles the oracle's C restatements (oracle/sparsity.c) with gcc into
oracle/_ref/liboracle.so.  The reference itself cannot be compiled here: its
only native parts are a Cython extension that needs PETSc headers and
libraries (pyop2/sparsity.pyx, setup.py:124-151) and loopy-generated wrappers
that need loopy; neither is installed, so nothing of the reference is built.
"""
import ctypes
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(REF_DIR, "liboracle.so")

_lib = None


def build(force=False):
    os.makedirs(REF_DIR, exist_ok=True)
    src = os.path.join(HERE, "sparsity.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        cmd = ["gcc", "-std=gnu11", "-O2", "-fPIC", "-shared", src, "-o", LIB + ".tmp"]
        subprocess.run(cmd, check=True)
        os.replace(LIB + ".tmp", LIB)
    return LIB


def liboracle():
    global _lib
    if _lib is None:
        build()
        _lib = ctypes.CDLL(LIB)
        _lib.oracle_sparsity_build.restype = ctypes.c_int
        _lib.oracle_free.restype = None
    return _lib


if __name__ == "__main__":
    print(build(force=True))
