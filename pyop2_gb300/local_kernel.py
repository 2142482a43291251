"""Local kernels (pyop2/local_kernel.py:30-207).

A local kernel is the user's C function, executed once per iteration entity.
Here it is compiled by NVRTC as a ``__device__`` function inside the
generated wrapper (see csrc/op2g_codegen.cpp), so the same C source runs on
the GPU unchanged.  Loopy kernels are not supported (there is no loopy).
"""
import hashlib

from pyop2_gb300.exceptions import NameTypeError
from pyop2_gb300.utils import validate_type


class LocalKernel:
    """User kernel: ``code`` defines a function called ``name``.

    Keyword arguments are those of the reference; ``cpp`` is accepted (the
    source is always compiled as CUDA C++), ``headers`` are prepended,
    ``flop_count`` is recorded for reporting.  ``user_code`` (host code run
    once per wrapper call) and ``ldargs`` have no meaning on the device and
    are rejected if non-empty.
    """

    @validate_type(("name", str, NameTypeError))
    def __init__(self, code, name, accesses=None, *, cpp=False, flop_count=None, headers=(),
                 include_dirs=(), ldargs=(), opts=None, requires_zeroed_output_arguments=False,
                 user_code="", events=()):
        if user_code:
            raise NotImplementedError("Kernel user_code runs on the host in the reference; "
                                      "it has no device equivalent")
        self.code = code
        self.name = name
        self.accesses = accesses
        self.cpp = cpp
        self.flop_count = flop_count
        self.headers = tuple(headers)
        self.include_dirs = tuple(include_dirs)
        self.ldargs = tuple(ldargs)
        self.opts = opts or {}
        self.requires_zeroed_output_arguments = requires_zeroed_output_arguments
        self.user_code = user_code
        self.events = events

    @property
    def source(self):
        """Full C source handed to NVRTC (headers first)."""
        return "\n".join(list(self.headers) + [self.code])

    @property
    def _code_key(self):
        key = (self.source, self.name, self.cpp, self.requires_zeroed_output_arguments)
        return hashlib.sha256(repr(key).encode()).hexdigest()

    @property
    def cache_key(self):
        return self._code_key, self.accesses, self.dtypes

    def __str__(self):
        return "OP2 Kernel: %s" % self.name

    def __repr__(self):
        return 'Kernel("""%s""", %r)' % (self.code, self.name)


class CStringLocalKernel(LocalKernel):
    """A LocalKernel from a string of C code."""

    @validate_type(("code", str, TypeError))
    def __init__(self, code, name, accesses=None, dtypes=None, **kwargs):
        super().__init__(code, name, accesses, **kwargs)
        self._dtypes = dtypes

    @property
    def dtypes(self):
        return self._dtypes

    @dtypes.setter
    def dtypes(self, dtypes):
        self._dtypes = dtypes


@validate_type(("name", str, NameTypeError))
def Kernel(code, name, **kwargs):
    """Construct a local kernel from C source (pyop2/local_kernel.py:30-41)."""
    if isinstance(code, str):
        return CStringLocalKernel(code, name, **kwargs)
    raise TypeError("code argument is the wrong type (only C source strings are supported)")
