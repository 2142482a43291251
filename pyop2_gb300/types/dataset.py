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
    """A tuple of DataSets (container only)."""

    def __init__(self, arg, dims=None):
        sets = tuple(arg)
        if dims is None:
            self._dsets = tuple(s if isinstance(s, DataSet) else s ** 1 for s in sets)
        else:
            dims = dims if isinstance(dims, (tuple, list)) else (dims,) * len(sets)
            self._dsets = tuple(s ** d for s, d in zip(sets, dims))
        self._set = None
        self._initialized = True
        self._name = "mdset_#x%x" % id(self)
        self.comm = None

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
