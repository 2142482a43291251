"""Globals (pyop2/types/glob.py:208-433): small values read or reduced by a
par_loop.  INC / MIN / MAX reductions happen on the device into the Global's
own device copy, so successive loops accumulate as in the reference
(pyop2/parloop.py:449-452)."""
import operator

import numpy as np

from pyop2_gb300 import exceptions as ex
from pyop2_gb300 import utils
from pyop2_gb300.configuration import configuration
from pyop2_gb300.device import Mirror
from pyop2_gb300.types.access import Access
from pyop2_gb300.types.dat import DataCarrier


def _global_arg(*args):
    """GlobalLegacyArg(*args), bound on first use (parloop imports this module)."""
    global _global_arg
    from pyop2_gb300.parloop import GlobalLegacyArg
    _global_arg = GlobalLegacyArg
    return GlobalLegacyArg(*args)


class Global(DataCarrier):
    """``Global(dim, data=None, dtype=None, name=None, comm=None)``."""

    _modes = [Access.READ, Access.INC, Access.MIN, Access.MAX]

    @utils.validate_type(('name', str, ex.NameTypeError))
    def __init__(self, dim, data=None, dtype=None, name=None, comm=None):
        if isinstance(dim, Global):
            src = dim
            self.__init__(src._dim, src.data_ro.copy(), dtype=src.dtype,
                          name="copy_of_%s" % src.name, comm=comm or src.comm)
            return
        self._dim = utils.as_tuple(dim, int)
        self._cdim = int(np.prod(self._dim))
        if data is None:
            self._dtype = np.dtype(dtype if dtype is not None else np.float64)
            arr = np.zeros(self._dim, dtype=self._dtype)
        else:
            arr = utils.verify_reshape(data, dtype, self._dim, allow_none=True)
            self._dtype = arr.dtype
            arr = np.array(arr, copy=True)
        self._m = Mirror(self._dtype, self._dim, arr)
        self._name = name or "global_#x%x" % id(self)
        self.comm = comm
        self._version = 0

    # the reference's validate_in access check written out, with its message
    # (this runs for every Global argument of every par_loop call)
    def __call__(self, access, map_=None):
        if configuration["type_check"] and access not in self._modes:
            raise ex.ModeValueError("access must be one of %s, not %r" % (self._modes, access))
        assert map_ is None
        return _global_arg(self, access)

    def __getitem__(self, idx):
        if idx != 0:
            raise ex.IndexValueError("Can only extract component 0 from %r" % self)
        return self

    def __iter__(self):
        yield self

    def __len__(self):
        return 1

    @property
    def dim(self):
        return self._dim

    @property
    def cdim(self):
        return self._cdim

    @property
    def shape(self):
        return self._dim

    @property
    def dtype(self):
        return self._dtype

    @property
    def name(self):
        return self._name

    @property
    def split(self):
        return (self,)

    @property
    def nbytes(self):
        return self.dtype.itemsize * self._cdim

    @property
    def data(self):
        self.increment_dat_version()
        d = self._m.host(write=True)
        if len(d) == 0:
            raise RuntimeError("Illegal access: No data associated with this Global!")
        return d

    @data.setter
    def data(self, value):
        self.increment_dat_version()
        self._m.host(write=True)[:] = utils.verify_reshape(value, self.dtype, self.dim)

    @property
    def data_ro(self):
        v = self._m.host(write=False).view()
        v.setflags(write=False)
        return v

    @property
    def data_wo(self):
        return self.data

    data_with_halos = data
    data_ro_with_halos = data_ro
    data_wo_with_halos = data_wo

    @property
    def halo_valid(self):
        return True

    @halo_valid.setter
    def halo_valid(self, v):
        pass

    @property
    def tensor(self):
        return self._m.tensor()

    def _device_ptr(self):
        return self._m.dev().data_ptr()

    def zero(self, subset=None):
        assert subset is None
        self.increment_dat_version()
        self._m.zero()

    def copy(self, other, subset=None):
        other.data = np.copy(self.data_ro)

    def duplicate(self):
        return type(self)(self.dim, data=np.copy(self.data_ro), dtype=self.dtype, name=self.name,
                          comm=self.comm)

    # ---- arithmetic on the (small) values, on the host
    # (pyop2/types/glob.py:132-204)
    def _op(self, other, op):
        ret = type(self)(self.dim, dtype=self.dtype, name=self.name, comm=self.comm)
        ret.data[:] = op(self.data_ro, other.data_ro if isinstance(other, Global) else other)
        return ret

    def _iop(self, other, op):
        op(self.data[:], other.data_ro if isinstance(other, Global) else other)
        return self

    def __pos__(self):
        return self.duplicate()

    def __neg__(self):
        return type(self)(self.dim, data=-np.copy(self.data_ro), dtype=self.dtype,
                          name=self.name, comm=self.comm)

    def __add__(self, other):
        return self._op(other, operator.add)

    def __radd__(self, other):
        return self + other

    def __sub__(self, other):
        return self._op(other, operator.sub)

    def __rsub__(self, other):
        ret = -self
        ret += other
        return ret

    def __mul__(self, other):
        return self._op(other, operator.mul)

    def __rmul__(self, other):
        return self.__mul__(other)

    def __truediv__(self, other):
        return self._op(other, operator.truediv)

    def __iadd__(self, other):
        return self._iop(other, operator.iadd)

    def __isub__(self, other):
        return self._iop(other, operator.isub)

    def __imul__(self, other):
        return self._iop(other, operator.imul)

    def __itruediv__(self, other):
        return self._iop(other, operator.itruediv)

    def inner(self, other):
        assert issubclass(type(other), type(self))
        return np.dot(self.data_ro, np.conj(other.data_ro))

    def __str__(self):
        return "OP2 Global Argument: %s with dim %s and value %s" % (self._name, self._dim,
                                                                    self.data_ro)

    def __repr__(self):
        return "Global(%r, %r, %r, %r)" % (self._dim, self.data_ro, self.dtype, self._name)


class Constant(Global):
    """A Global that par_loops may only READ (pyop2/types/glob.py:371-433)."""

    _modes = [Access.READ]

    @utils.validate_in(('access', _modes, ex.ModeValueError))
    def __call__(self, access, map_=None):
        from pyop2_gb300.parloop import GlobalLegacyArg
        return GlobalLegacyArg(self, access)
