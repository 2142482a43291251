"""DataSets (pyop2/types/dataset.py:16-195): a Set plus a per-entity shape."""
import numbers

import numpy as np

from pyop2_gb300 import exceptions as ex
from pyop2_gb300 import utils
from pyop2_gb300.types.set import ExtrudedSet, Set, Subset


class DataSet:
    """Shape ``dim`` of the values held on each entity of ``iter_set``.

    Instances are cached per (set, dim), as the reference's ObjectCached
    DataSet is, so ``s ** 2 is s ** 2``.
    """

    def __new__(cls, iter_set, dim=1, name=None):
        if cls is DataSet and isinstance(iter_set, Set) and not isinstance(iter_set, (ExtrudedSet, Subset)):
            key = ("DataSet", utils.as_tuple(dim, numbers.Integral) if not isinstance(dim, numbers.Integral) else (dim,))
            cached = iter_set._cache.get(key)
            if cached is not None:
                return cached
            obj = super().__new__(cls)
            obj._initialized = False
            iter_set._cache[key] = obj
            return obj
        obj = super().__new__(cls)
        obj._initialized = False
        return obj

    @utils.validate_type(('iter_set', Set, ex.SetTypeError),
                         ('dim', (numbers.Integral, tuple, list), ex.DimTypeError),
                         ('name', str, ex.NameTypeError))
    def __init__(self, iter_set, dim=1, name=None):
        if isinstance(iter_set, ExtrudedSet) and not isinstance(iter_set, Subset):
            raise NotImplementedError("Not allowed!")
        if self._initialized:
            return
        if isinstance(iter_set, Subset):
            raise NotImplementedError("Deriving a DataSet from a Subset is unsupported")
        self.comm = iter_set.comm
        self._set = iter_set
        self._dim = utils.as_tuple(dim, numbers.Integral)
        self._cdim = int(np.prod(self._dim))
        self._name = name or "dset_#x%x" % id(self)
        self._initialized = True

    def __getattr__(self, name):
        if name.startswith("__") or name in ("_set", "_initialized"):
            raise AttributeError(name)
        return getattr(self._set, name)

    def __getitem__(self, idx):
        assert idx == 0
        return self

    @property
    def dim(self):
        return self._dim

    @property
    def cdim(self):
        return self._cdim

    @property
    def name(self):
        return self._name

    @property
    def set(self):
        return self._set

    def __iter__(self):
        yield self

    def __len__(self):
        return 1

    def __str__(self):
        return "OP2 DataSet: %s on set %s, with dim %s" % (self._name, self._set, self._dim)

    def __repr__(self):
        return "DataSet(%r, %r, %r)" % (self._set, self._dim, self._name)

    def __contains__(self, dat):
        return dat.dataset == self


class GlobalDataSet(DataSet):
    """DataSet of a Global."""

    def __init__(self, global_):
        self._global = global_
        self._set = None
        self._dim = global_.dim
        self._cdim = global_.cdim
        self._name = "gdset_#x%x" % id(self)
        self._initialized = True
        self.comm = None

    @property
    def set(self):
        from pyop2_gb300.types.set import GlobalSet
        return GlobalSet()


class MixedDataSet(DataSet):
    """A tuple of DataSets (pyop2/types/dataset.py:304-460).

    ``MixedDataSet(mset_or_sets, dims)`` with one dim or one per set, or
    ``MixedDataSet(iterable of DataSets and/or Sets)`` (Sets become dim 1).
    Cached per tuple of component DataSets.
    """

    def __new__(cls, arg, dims=None):
        dsets = cls._process_args(arg, dims)
        key = ("MixedDataSet", dsets)
        holder = dsets[0].set._cache
        obj = holder.get(key)
        if obj is None:
            obj = object.__new__(cls)
            obj._initialized = False
            obj._pending = dsets
            holder[key] = obj
        return obj

    @staticmethod
    def _process_args(arg, dims=None):
        from pyop2_gb300.types.set import MixedSet
        if dims is not None:
            sets = arg.split if isinstance(arg, MixedSet) else tuple(arg)
            dims = (dims,) * len(sets) if isinstance(dims, numbers.Integral) else tuple(dims)
            if len(sets) != len(dims):
                raise ValueError("Got MixedSet of %d Sets but %s dims" % (len(sets), len(dims)))
            return tuple(s ** d for s, d in zip(sets, dims))
        out = tuple(s if isinstance(s, DataSet) else s ** 1 for s in arg)
        for d in out:
            if not isinstance(d, DataSet):
                raise TypeError("MixedDataSet components must be DataSets or Sets")
        return out

    def __init__(self, arg, dims=None):
        if self._initialized:
            return
        self._dsets = self._pending
        self._set = None
        self._name = "mdset_#x%x" % id(self)
        self.comm = None
        self._initialized = True

    def __getattr__(self, name):
        raise AttributeError(name)

    def __getitem__(self, idx):
        return self._dsets[idx]

    def __iter__(self):
        yield from self._dsets

    def __len__(self):
        return len(self._dsets)

    @property
    def split(self):
        return self._dsets

    @property
    def dim(self):
        return tuple(s.dim for s in self._dsets)

    @property
    def cdim(self):
        return sum(s.cdim for s in self._dsets)

    @property
    def name(self):
        return tuple(s.name for s in self._dsets)

    @property
    def set(self):
        from pyop2_gb300.types.set import MixedSet
        return MixedSet(s.set for s in self._dsets)

    @property
    def size(self):
        return sum(s.size for s in self._dsets)

    @property
    def total_size(self):
        return sum(s.total_size for s in self._dsets)

    @property
    def offsets(self):
        """Start of each component in the concatenated dof numbering."""
        o = [0]
        for s in self._dsets:
            o.append(o[-1] + s.size * s.cdim)
        return tuple(o)

    def __contains__(self, dat):
        return dat.dataset == self

    def __str__(self):
        return "OP2 MixedDataSet composed of DataSets: %s" % (self._dsets,)

    def __repr__(self):
        return "MixedDataSet(%r)" % (self._dsets,)
