"""Dats (pyop2/types/dat.py:25-784): per-entity data held in HBM.

Storage is ``(dataset.total_size,) + dim`` C-contiguous (pyop2/types/dat.py:81)
in a device buffer with a lazily synchronised host mirror.  ``data`` /
``data_ro`` / ``data_wo`` (and the ``_with_halos`` variants) have the
reference's meaning; reading them after a par_loop copies the device data
back once.
"""
import numpy as np

from pyop2_gb300 import exceptions as ex
from pyop2_gb300 import utils
from pyop2_gb300.configuration import configuration
from pyop2_gb300.datatypes import ScalarType
from pyop2_gb300.device import Mirror
from pyop2_gb300.types.access import Access
from pyop2_gb300.types.dataset import DataSet
from pyop2_gb300.types.set import ExtrudedSet, Set


class DataCarrier:
    """Common base of Dat, Global and Mat (pyop2/types/data_carrier.py:13-48)."""

    _version = 0

    def increment_dat_version(self):
        self._version += 1

    @property
    def dat_version(self):
        return self._version

    @property
    def ctype(self):
        from pyop2_gb300.datatypes import as_cstr
        return as_cstr(self.dtype)


def _dat_arg(*args):
    """DatLegacyArg(*args), bound on first use (parloop imports this module)."""
    global _dat_arg
    from pyop2_gb300.parloop import DatLegacyArg
    _dat_arg = DatLegacyArg
    return DatLegacyArg(*args)


class AbstractDat(DataCarrier):
    _modes = [Access.READ, Access.WRITE, Access.RW, Access.INC, Access.MIN, Access.MAX]


class Dat(AbstractDat):
    """OP2 vector data: values on every entity of a DataSet.

    ``Dat(set_or_dataset, data=None, dtype=None, name=None)``; a Set means a
    dim-1 DataSet, a Dat means a copy; missing data is zero.
    """

    @utils.validate_type(('dataset', (DataCarrier, DataSet, Set), ex.DataSetTypeError),
                         ('name', str, ex.NameTypeError))
    @utils.validate_dtype(('dtype', None, ex.DataTypeError))
    def __init__(self, dataset, data=None, dtype=None, name=None):
        if isinstance(dataset, Dat):
            src = dataset
            self.__init__(src.dataset, None, dtype=src.dtype, name="copy_of_%s" % src.name)
            src.copy(self)
            return
        if type(dataset) is Set or type(dataset) is ExtrudedSet:
            dataset = dataset ** 1
        self._dataset = dataset
        self.comm = dataset.comm
        self._shape = (dataset.total_size,) + (() if dataset.cdim == 1 else dataset.dim)
        if data is None:
            self._dtype = np.dtype(dtype if dtype is not None else ScalarType)
            self._m = Mirror(self._dtype, self._shape)
        else:
            arr = utils.verify_reshape(data, dtype, self._shape, allow_none=True)
            if arr.size == 0 and int(np.prod(self._shape)) != 0:
                raise ex.DataValueError("Invalid data: expected %d values" % int(np.prod(self._shape)))
            self._dtype = arr.dtype
            self._m = Mirror(self._dtype, self._shape, np.array(arr, copy=True))
        self._name = name or "dat_#x%x" % id(self)
        self.halo_valid = True
        self._version = 0

    # ---- kernel-argument construction (runs for every argument of every
    # par_loop call, so the reference's validate_in access check is written
    # out here, with its message)
    def __call__(self, access, path=None):
        if configuration["type_check"]:
            if access not in AbstractDat._modes:
                raise ex.ModeValueError("access must be one of %s, not %r"
                                        % (AbstractDat._modes, access))
            if path is not None and path.toset != self.dataset.set:
                raise ex.MapValueError("To Set of Map does not match Set of Dat.")
        return _dat_arg(self, path, access)

    def __getitem__(self, idx):
        if idx != 0:
            raise ex.IndexValueError("Can only extract component 0 from %r" % self)
        return self

    @property
    def split(self):
        return (self,)

    @property
    def dataset(self):
        return self._dataset

    @property
    def dim(self):
        return self.dataset.dim

    @property
    def cdim(self):
        return self.dataset.cdim

    @property
    def shape(self):
        return self._shape

    @property
    def dtype(self):
        return self._dtype

    @property
    def name(self):
        return self._name

    @property
    def nbytes(self):
        return self.dtype.itemsize * self.dataset.total_size * self.dataset.cdim

    # ---- host accessors
    @property
    def data(self):
        """Writable host view of the owned values (marks the host newer)."""
        self.increment_dat_version()
        self.halo_valid = False
        v = self._m.host(write=True)[:self.dataset.size].view()
        v.setflags(write=True)
        return v

    @property
    def data_with_halos(self):
        self.increment_dat_version()
        self.halo_valid = False
        v = self._m.host(write=True).view()
        v.setflags(write=True)
        return v

    @property
    def data_ro(self):
        v = self._m.host(write=False)[:self.dataset.size].view()
        v.setflags(write=False)
        return v

    @property
    def data_ro_with_halos(self):
        v = self._m.host(write=False).view()
        v.setflags(write=False)
        return v

    @property
    def data_wo(self):
        return self.data

    @property
    def data_wo_with_halos(self):
        return self.data_with_halos

    @property
    def _is_allocated(self):
        """True once a host buffer exists (storage is allocated lazily)."""
        return self._m.host_allocated()

    @property
    def _data(self):
        """The full host array including ghost entries."""
        return self._m.host(write=False)

    @_data.setter
    def _data(self, value):
        """Overwrite every value, ghosts included (the reference's tests
        assign ``dat._data`` directly)."""
        self.increment_dat_version()
        self._m.host(write=True)[...] = np.asarray(value).reshape(self._shape)

    # ---- device access
    @property
    def tensor(self):
        """The device values as a torch tensor of shape ``shape`` (no copy).
        Writes through this view must be followed by ``mark_device_modified``."""
        return self._m.tensor().view(self._shape)

    def mark_device_modified(self):
        self._m.dev_modified()
        self.increment_dat_version()

    def _device_ptr(self):
        return self._m.dev().data_ptr()

    @classmethod
    def from_tensor(cls, dataset, tensor, name=None):
        """A Dat whose device storage is ``tensor`` (CUDA, contiguous, matching
        shape and dtype), without copying.  The Dat writes into the tensor."""
        import torch
        from pyop2_gb300 import device
        if type(dataset) is Set:
            dataset = dataset ** 1
        d = cls.__new__(cls)
        d._dataset = dataset
        d.comm = dataset.comm
        d._shape = (dataset.total_size,) + (() if dataset.cdim == 1 else dataset.dim)
        if not tensor.is_cuda or not tensor.is_contiguous():
            raise ValueError("from_tensor needs a contiguous CUDA tensor")
        if tuple(tensor.shape) != d._shape and tensor.numel() != int(np.prod(d._shape)):
            raise ValueError("tensor shape %s does not match %s" % (tuple(tensor.shape), d._shape))
        npdt = {torch.float64: np.float64, torch.float32: np.float32,
                torch.int32: np.int32, torch.int64: np.int64}[tensor.dtype]
        d._dtype = np.dtype(npdt)
        d._m = Mirror(d._dtype, d._shape)
        d._m._dev = tensor.view(-1).view(torch.uint8)
        d._m.state = "device"
        d._name = name or "dat_#x%x" % id(d)
        d.halo_valid = True
        d._version = 0
        device.require()
        return d

    def _rebind(self, tensor):
        """Make ``tensor`` (CUDA, contiguous, same element count and dtype)
        this Dat's device storage, without copying: a loop built on this Dat
        then runs on the tensor (it re-reads the pointer at launch)."""
        import torch
        if not tensor.is_cuda or not tensor.is_contiguous():
            raise ValueError("_rebind needs a contiguous CUDA tensor")
        if tensor.numel() != int(np.prod(self._shape)) or \
                tensor.element_size() != self._dtype.itemsize:
            raise ValueError("tensor does not match the Dat's shape and dtype")
        self._m._dev = tensor.view(-1).view(torch.uint8)
        self._m._host = None
        self._m.state = "device"
        self.increment_dat_version()

    # ---- operations
    def zero(self, subset=None):
        self.increment_dat_version()
        if subset is None:
            self._m.zero()
            self.halo_valid = True
        elif subset.superset != self.dataset.set:
            raise ex.MapValueError("The subset and dataset are incompatible")
        else:
            self.data[subset.owned_indices] = 0

    def copy(self, other, subset=None):
        if other is self:
            return
        if subset is None:
            other.data_with_halos[:] = self.data_ro_with_halos
            other.halo_valid = True
        elif subset.superset != self.dataset.set:
            raise ex.MapValueError("The subset and dataset are incompatible")
        else:
            other.data[subset.owned_indices] = self.data_ro[subset.owned_indices]

    def save(self, filename):
        """Write the owned values to ``filename`` in NumPy format."""
        np.save(filename, self.data_ro)

    def load(self, filename):
        if filename[-4:] != ".npy":
            filename = filename + ".npy"
        self.data[:] = np.load(filename)

    # ---- pointwise linear algebra (pyop2/types/dat.py:343-574), executed
    # as generated direct par_loops over the owned entities, as the
    # reference does
    _kernel_cache = {}

    def _kernel(self, key, body, name):
        from pyop2_gb300.local_kernel import Kernel
        k = Dat._kernel_cache.get(key)
        if k is None:
            k = Dat._kernel_cache[key] = Kernel(body, name)
        return k

    def _other(self, other):
        from pyop2_gb300.types.glob import Global
        if isinstance(other, Dat):
            self._check_shape(other)
            return other, False
        return Global(1, data=other, dtype=self.dtype), True

    def _check_shape(self, other):
        if other.dataset.dim != self.dataset.dim:
            raise ValueError("Mismatched shapes in operands %s and %s"
                             % (self.dataset.dim, other.dataset.dim))

    def _op(self, other, op, opname):
        from pyop2_gb300.datatypes import as_cstr
        from pyop2_gb300.parloop import run_once as par_loop
        from pyop2_gb300.types.access import READ, WRITE
        o, scalar = self._other(other)
        t, to = as_cstr(self.dtype), as_cstr(o.dtype)
        name = "op2g_dat_%s" % opname
        key = ("op", opname, scalar, self.cdim, t, to)
        k = self._kernel(key, "static void %s(const %s *a, const %s *b, %s *r) "
                         "{ for (int i = 0; i < %d; ++i) r[i] = a[i] %s b[%s]; }"
                         % (name, t, to, t, self.cdim, op, "0" if scalar else "i"), name)
        ret = Dat(self.dataset, None, self.dtype)
        par_loop(k, self.dataset.set, self(READ), o(READ), ret(WRITE))
        return ret

    def _iop(self, other, op, opname):
        from pyop2_gb300.datatypes import as_cstr
        from pyop2_gb300.parloop import run_once as par_loop
        from pyop2_gb300.types.access import READ, RW
        o, scalar = self._other(other)
        t, to = as_cstr(self.dtype), as_cstr(o.dtype)
        name = "op2g_dat_i%s" % opname
        key = ("iop", opname, scalar, self.cdim, t, to)
        k = self._kernel(key, "static void %s(%s *a, const %s *b) "
                         "{ for (int i = 0; i < %d; ++i) a[i] %s= b[%s]; }"
                         % (name, t, to, self.cdim, op, "0" if scalar else "i"), name)
        if o is self:
            o = Dat(self)
        par_loop(k, self.dataset.set, self(RW), o(READ))
        return self

    def __add__(self, other):
        return self._op(other, "+", "add")

    def __radd__(self, other):
        return self + other

    def __sub__(self, other):
        return self._op(other, "-", "sub")

    def __rsub__(self, other):
        ret = -self
        ret += other
        return ret

    def __mul__(self, other):
        return self._op(other, "*", "mul")

    def __rmul__(self, other):
        return self * other

    def __truediv__(self, other):
        return self._op(other, "/", "div")

    def __iadd__(self, other):
        return self._iop(other, "+", "add")

    def __isub__(self, other):
        return self._iop(other, "-", "sub")

    def __imul__(self, other):
        return self._iop(other, "*", "mul")

    def __itruediv__(self, other):
        return self._iop(other, "/", "div")

    def __pos__(self):
        return Dat(self)

    def __neg__(self):
        from pyop2_gb300.datatypes import as_cstr
        from pyop2_gb300.parloop import run_once as par_loop
        from pyop2_gb300.types.access import READ, WRITE
        t = as_cstr(self.dtype)
        k = self._kernel(("neg", self.cdim, t),
                         "static void op2g_dat_neg(const %s *a, %s *r) "
                         "{ for (int i = 0; i < %d; ++i) r[i] = -a[i]; }" % (t, t, self.cdim),
                         "op2g_dat_neg")
        ret = Dat(self.dataset, None, self.dtype)
        par_loop(k, self.dataset.set, self(READ), ret(WRITE))
        return ret

    def inner(self, other):
        """Euclidean inner product over the owned entities (a Global INC
        reduction on the device)."""
        from pyop2_gb300.datatypes import as_cstr
        from pyop2_gb300.parloop import run_once as par_loop
        from pyop2_gb300.types.access import INC, READ
        from pyop2_gb300.types.glob import Global
        self._check_shape(other)
        t = as_cstr(self.dtype)
        k = self._kernel(("inner", self.cdim, t),
                         "static void op2g_dat_inner(const %s *a, const %s *b, %s *r) "
                         "{ for (int i = 0; i < %d; ++i) r[0] += a[i] * b[i]; }"
                         % (t, t, t, self.cdim), "op2g_dat_inner")
        ret = Global(1, data=0, dtype=self.dtype)
        par_loop(k, self.dataset.set, self(READ), other(READ), ret(INC))
        return ret.data_ro[0]

    @property
    def norm(self):
        """The l2 norm of the owned values."""
        from math import sqrt
        return sqrt(self.inner(self))

    def __iter__(self):
        yield self

    def __len__(self):
        return 1

    def __str__(self):
        return "OP2 Dat: %s on (%s) with datatype %s" % (self._name, self._dataset, self.dtype.name)

    def __repr__(self):
        return "Dat(%r, None, %r, %r)" % (self._dataset, self.dtype, self._name)

    # ---- vector views (pyop2/types/dat.py:762-784 hand out a PETSc Vec; here
    # the Vec is the flat device tensor of the owned values)
    def vec_context(self, access):
        """Context manager yielding the owned values as a flat CUDA tensor;
        unless ``access`` is READ the Dat counts as modified on exit."""
        return _VecContext(self, access)

    @property
    def vec(self):
        return self.vec_context(Access.RW)

    @property
    def vec_wo(self):
        return self.vec_context(Access.WRITE)

    @property
    def vec_ro(self):
        return self.vec_context(Access.READ)

    # ---- halo freezing (pyop2/types/dat.py:634-665, 1154-1175).  A single
    # device has no halo exchanges to skip, but the bookkeeping is kept: a Dat
    # frozen for one access mode may only be used with that mode.
    _halo_frozen = False
    _frozen_access_mode = None

    def freeze_halo(self, access_mode):
        if self._halo_frozen:
            raise RuntimeError("Expected an unfrozen halo")
        self._halo_frozen = True
        self._frozen_access_mode = access_mode

    def unfreeze_halo(self):
        if not self._halo_frozen:
            raise RuntimeError("Expected a frozen halo")
        self._halo_frozen = False
        self._frozen_access_mode = None

    def frozen_halo(self, access_mode):
        """Context manager: halo exchanges off, accesses restricted to
        ``access_mode`` while it is active."""
        return _FrozenHalo(self, access_mode)

    # halo operations are no-ops on one device (no MPI halos)
    def global_to_local_begin(self, access_mode):
        pass

    def global_to_local_end(self, access_mode):
        pass

    def local_to_global_begin(self, insert_mode):
        pass

    def local_to_global_end(self, insert_mode):
        pass


class DatView(Dat):
    """One component of a Dat (pyop2/types/dat.py:668-760): in a par_loop the
    kernel sees only component ``index``, with dim 1; ``data`` and friends
    are the matching column of the parent's arrays.  No storage of its own:
    the device pointer is the parent's, advanced to the component, and the
    wrapper strides by the parent's dim."""

    def __init__(self, dat, index):
        index = utils.as_tuple(index)
        assert len(index) == len(dat.dim)
        for i, d in zip(index, dat.dim):
            if not (0 <= i < d):
                raise ex.IndexValueError("Can't create DatView with index %s for Dat with "
                                         "shape %s" % (index, dat.dim))
        self.index = index
        self._idx = (slice(None), *index)
        self._parent = dat
        self._dataset = dat.dataset
        self.comm = dat.comm
        self._dtype = dat.dtype
        self._m = dat._m
        self._shape = (dat.dataset.total_size,)
        self._name = "view[%s](%s)" % (index, dat.name)
        # flat position of the component inside one entity's values
        self._view_offset = int(np.ravel_multi_index(index, dat.dim)) if dat.cdim > 1 else 0
        self._view_stride = dat.cdim

    @property
    def cdim(self):
        return 1

    @property
    def dim(self):
        return (1,)

    @property
    def halo_valid(self):
        return self._parent.halo_valid

    @halo_valid.setter
    def halo_valid(self, value):
        self._parent.halo_valid = value

    @property
    def dat_version(self):
        return self._parent.dat_version

    def increment_dat_version(self):
        self._parent.increment_dat_version()

    @property
    def _halo_frozen(self):
        return self._parent._halo_frozen

    @property
    def _frozen_access_mode(self):
        return self._parent._frozen_access_mode

    @property
    def _data(self):
        return self._parent._data[self._idx]

    @property
    def data(self):
        return self._parent.data[self._idx]

    @property
    def data_ro(self):
        return self._parent.data_ro[self._idx]

    @property
    def data_wo(self):
        return self._parent.data_wo[self._idx]

    @property
    def data_with_halos(self):
        return self._parent.data_with_halos[self._idx]

    @property
    def data_ro_with_halos(self):
        return self._parent.data_ro_with_halos[self._idx]

    @property
    def data_wo_with_halos(self):
        return self._parent.data_wo_with_halos[self._idx]

    @property
    def nbytes(self):
        return self.dtype.itemsize * self.dataset.total_size

    @property
    def tensor(self):
        """Strided device view of the component."""
        t = self._parent.tensor
        return t.reshape(t.shape[0], -1)[:, self._view_offset]

    def _device_ptr(self):
        return self._m.dev().data_ptr() + self._view_offset * self.dtype.itemsize

    def mark_device_modified(self):
        self._parent.mark_device_modified()

    def zero(self, subset=None):
        if subset is not None:
            self.data[subset.owned_indices] = 0
            return
        self.increment_dat_version()
        self.tensor.zero_()
        self._m.dev_modified()
        self._parent.halo_valid = True

    def __repr__(self):
        return "DatView(%r, %r)" % (self._parent, self.index)

    def __str__(self):
        return "OP2 DatView: %s of %s" % (self.index, self._parent)


class _VecContext:
    """``with dat.vec as v:``: ``v`` is the flat device tensor of the owned
    values (a MixedDat's components concatenated, copied back on exit)."""

    def __init__(self, dat, access):
        self._dat = dat
        self._access = access

    def __enter__(self):
        import torch
        d = self._dat
        if isinstance(d, MixedDat):
            self._parts = [c.tensor[:c.dataset.size].reshape(-1) for c in d]
            self._v = torch.cat(self._parts)
        else:
            self._v = d.tensor[:d.dataset.size].reshape(-1)
        self._before = self._v.clone() if self._access is not Access.READ else None
        return self._v

    def __exit__(self, *args):
        if self._access is Access.READ:
            return
        d = self._dat
        if isinstance(d, MixedDat):
            o = 0
            for c, part in zip(d, self._parts):
                n = part.numel()
                if not bool((self._v[o:o + n] == self._before[o:o + n]).all()):
                    part.copy_(self._v[o:o + n])
                    c.mark_device_modified()
                    c.halo_valid = False
                o += n
        elif not bool((self._v == self._before).all()):
            d.mark_device_modified()
            d.halo_valid = False


class _FrozenHalo:
    """``with dat.frozen_halo(mode):`` (pyop2/types/dat.py:1154-1175)."""

    def __init__(self, dat, access_mode):
        self._dat = dat
        self._access_mode = access_mode

    def __enter__(self):
        self._dat.global_to_local_begin(self._access_mode)
        self._dat.global_to_local_end(self._access_mode)
        self._dat.freeze_halo(self._access_mode)

    def __exit__(self, *args):
        self._dat.unfreeze_halo()
        self._dat.local_to_global_begin(self._access_mode)
        self._dat.local_to_global_end(self._access_mode)


class MixedDat(AbstractDat):
    """A tuple of Dats over the components of a MixedDataSet
    (pyop2/types/dat.py:787-1151).

    ``MixedDat(mdset_or_sets_or_dats)``: a MixedDataSet, MixedSet or iterable
    of DataSets/Sets makes new zeroed Dats; an iterable of Dats is used as
    is; a MixedDat is copied.  ``mdat(access, mixed_map)`` hands the kernel
    one pack that concatenates the components' packs.
    """

    def __init__(self, mdset_or_dats):
        from pyop2_gb300.types.glob import Global

        def make(x):
            if isinstance(x, (Dat, Global)):
                return x
            if isinstance(x, (DataSet, Set)):
                return Dat(x)
            raise ex.DataSetTypeError("MixedDat components must be Dats, DataSets or Sets, "
                                      "not %r" % type(x))
        if isinstance(mdset_or_dats, MixedDat):
            self._dats = tuple(Dat(d) for d in mdset_or_dats)
        else:
            self._dats = tuple(make(d) for d in mdset_or_dats)
        if not all(d.dtype == self._dats[0].dtype for d in self._dats):
            raise ex.DataValueError("MixedDat with different dtypes is not supported")
        self.comm = None

    @utils.validate_in(('access', AbstractDat._modes, ex.ModeValueError))
    def __call__(self, access, path=None):
        from pyop2_gb300.parloop import MixedDatLegacyArg
        from pyop2_gb300.types.map import MixedMap
        if not isinstance(path, MixedMap):
            raise ex.MapTypeError("A MixedDat is accessed through a MixedMap")
        if len(path) != len(self._dats):
            raise ex.MapValueError("MixedMap has %d maps for %d Dats" % (len(path), len(self._dats)))
        for d, m in zip(self._dats, path):
            # the reference does not compare tosets here; a map reaching
            # past its Dat's storage is still refused (it would address
            # outside the device buffer)
            if m.toset.total_size > d.dataset.total_size:
                raise ex.MapValueError("Map %s reaches beyond Dat %s" % (m.name, d.name))
        return MixedDatLegacyArg(self, path, access)

    @property
    def dat_version(self):
        return sum(d.dat_version for d in self._dats)

    def increment_dat_version(self):
        for d in self._dats:
            d.increment_dat_version()

    def __getitem__(self, idx):
        return self._dats[idx]

    def __iter__(self):
        yield from self._dats

    def __len__(self):
        return len(self._dats)

    @property
    def split(self):
        return self._dats

    @property
    def dtype(self):
        return self._dats[0].dtype

    @property
    def dataset(self):
        from pyop2_gb300.types.dataset import MixedDataSet
        return MixedDataSet(tuple(d.dataset for d in self._dats))

    @property
    def dim(self):
        return tuple(d.dataset.dim for d in self._dats)

    @property
    def cdim(self):
        return sum(d.cdim for d in self._dats)

    def __hash__(self):
        return hash(self._dats)

    def __eq__(self, other):
        """MixedDats of the same Dats are equal (pyop2/types/dat.py:1007-1016)."""
        return type(self) is type(other) and self._dats == other._dats

    def __ne__(self, other):
        return not self.__eq__(other)

    @property
    def name(self):
        return tuple(d.name for d in self._dats)

    @property
    def nbytes(self):
        return int(sum(d.nbytes for d in self._dats))

    @property
    def data(self):
        return tuple(d.data for d in self._dats)

    @property
    def data_with_halos(self):
        return tuple(d.data_with_halos for d in self._dats)

    @property
    def data_ro(self):
        return tuple(d.data_ro for d in self._dats)

    @property
    def data_ro_with_halos(self):
        return tuple(d.data_ro_with_halos for d in self._dats)

    @property
    def data_wo(self):
        return tuple(d.data_wo for d in self._dats)

    @property
    def data_wo_with_halos(self):
        return tuple(d.data_wo_with_halos for d in self._dats)

    @property
    def _data(self):
        return tuple(d._data for d in self._dats)

    @property
    def halo_valid(self):
        return all(d.halo_valid for d in self._dats)

    @halo_valid.setter
    def halo_valid(self, val):
        for d in self._dats:
            d.halo_valid = val

    def zero(self, subset=None):
        if subset is not None:
            raise NotImplementedError("Subsets of mixed sets not implemented")
        for d in self._dats:
            d.zero()

    def copy(self, other, subset=None):
        if subset is not None:
            raise NotImplementedError("MixedDat.copy with a Subset is not supported")
        for s, o in zip(self, other):
            s.copy(o)

    def save(self, filename):
        """Write the components' owned values to ``filename`` as one NumPy
        array (components of one shape, as the reference's file format)."""
        np.save(filename, self.data_ro)

    def load(self, filename):
        if filename[-4:] != ".npy":
            filename = filename + ".npy"
        for d, v in zip(self._dats, np.load(filename)):
            d.data[:] = v

    def _check_shape(self, other):
        if tuple(d.dataset.dim for d in other) != tuple(d.dataset.dim for d in self):
            raise ValueError("Mismatched shapes in operands")

    def _op(self, other, fn):
        if np.isscalar(other):
            return MixedDat([fn(s, other) for s in self])
        self._check_shape(other)
        return MixedDat([fn(s, o) for s, o in zip(self, other)])

    def _iop(self, other, fn):
        if np.isscalar(other):
            for s in self:
                fn(s, other)
        else:
            self._check_shape(other)
            for s, o in zip(self, other):
                fn(s, o)
        return self

    def inner(self, other):
        return sum(s.inner(o) for s, o in zip(self, other))

    @property
    def norm(self):
        from math import sqrt
        return sqrt(self.inner(self))

    def __pos__(self):
        return MixedDat([+s for s in self])

    def __neg__(self):
        return MixedDat([-s for s in self])

    def __add__(self, other):
        return self._op(other, lambda a, b: a + b)

    def __radd__(self, other):
        return self._op(other, lambda a, b: b + a)

    def __sub__(self, other):
        return self._op(other, lambda a, b: a - b)

    def __rsub__(self, other):
        return self._op(other, lambda a, b: b - a)

    def __mul__(self, other):
        return self._op(other, lambda a, b: a * b)

    def __rmul__(self, other):
        return self._op(other, lambda a, b: b * a)

    def __truediv__(self, other):
        return self._op(other, lambda a, b: a / b)

    def __iadd__(self, other):
        return self._iop(other, lambda a, b: a.__iadd__(b))

    def __isub__(self, other):
        return self._iop(other, lambda a, b: a.__isub__(b))

    def __imul__(self, other):
        return self._iop(other, lambda a, b: a.__imul__(b))

    def __itruediv__(self, other):
        return self._iop(other, lambda a, b: a.__itruediv__(b))

    def __str__(self):
        return "OP2 MixedDat composed of Dats: %s" % (self._dats,)

    def __repr__(self):
        return "MixedDat(%r)" % (self._dats,)

    @property
    def _halo_frozen(self):
        return all(d._halo_frozen for d in self._dats)

    def vec_context(self, access):
        return _VecContext(self, access)

    @property
    def vec(self):
        return self.vec_context(Access.RW)

    @property
    def vec_wo(self):
        return self.vec_context(Access.WRITE)

    @property
    def vec_ro(self):
        return self.vec_context(Access.READ)

    def freeze_halo(self, access_mode):
        for d in self._dats:
            d.freeze_halo(access_mode)

    def unfreeze_halo(self):
        for d in self._dats:
            d.unfreeze_halo()

    def frozen_halo(self, access_mode):
        return _FrozenHalo(self, access_mode)

    def global_to_local_begin(self, access_mode):
        pass

    def global_to_local_end(self, access_mode):
        pass

    def local_to_global_begin(self, insert_mode):
        pass

    def local_to_global_end(self, insert_mode):
        pass
