"""Iteration sets (pyop2/types/set.py): Set :16-226, ExtrudedSet :305-391,
Subset :394-530, SetPartition :533-537, MixedSet :540-662."""
import numbers

import numpy as np

from pyop2_gb300 import exceptions as ex
from pyop2_gb300 import utils
from pyop2_gb300.datatypes import IntType
from pyop2_gb300.device import Mirror


class SetPartition:
    def __init__(self, set, offset, size):
        self.set = set
        self.offset = offset
        self.size = size


class Set:
    """An OP2 set of ``size`` entities, or sizes ``(core, owned, total)``.

    Only [0, size) is iterated; entities in [size, total_size) are ghosts
    that may be read through maps but are never executed.
    """

    _CORE_SIZE, _OWNED_SIZE, _GHOST_SIZE = 0, 1, 2
    _extruded = False
    _extruded_periodic = False

    @utils.validate_type(('size', (numbers.Integral, tuple, list, np.ndarray), ex.SizeTypeError),
                         ('name', str, ex.NameTypeError))
    def __init__(self, size, name=None, halo=None, comm=None, constrained_size=0):
        if isinstance(size, numbers.Integral):
            size = [size] * 3
        size = utils.as_tuple(size, numbers.Integral, 3)
        if not (size[0] <= size[1] <= size[2]):
            raise ex.SizeTypeError("Set received invalid sizes: %s" % (size,))
        self._sizes = tuple(int(s) for s in size)
        self._name = name or "set_#x%x" % id(self)
        self._halo = halo
        self.comm = comm
        self._constrained_size = constrained_size
        self._cache = {}
        self._partition_size = 1024

    @property
    def indices(self):
        return range(self.total_size)

    @property
    def core_size(self):
        return self._sizes[0]

    @property
    def size(self):
        return self._sizes[1]

    @property
    def total_size(self):
        return self._sizes[2]

    @property
    def sizes(self):
        return self._sizes

    @property
    def constrained_size(self):
        return self._constrained_size

    @property
    def core_part(self):
        return SetPartition(self, 0, self.core_size)

    @property
    def owned_part(self):
        return SetPartition(self, self.core_size, self.size - self.core_size)

    @property
    def name(self):
        return self._name

    @property
    def halo(self):
        return self._halo

    @property
    def partition_size(self):
        return self._partition_size

    @partition_size.setter
    def partition_size(self, v):
        self._partition_size = v

    @property
    def layers(self):
        """None: a plain Set is not extruded (pyop2/types/set.py:195-197)."""
        return None

    def __iter__(self):
        yield self

    def __getitem__(self, idx):
        if idx != 0:
            raise ex.IndexValueError("Can only extract component 0 from %r" % self)
        return self

    def __len__(self):
        return 1

    def __contains__(self, dset):
        """A DataSet is in the Set it was built on (pyop2/types/set.py:181-187)."""
        from pyop2_gb300.types.dataset import DataSet
        if isinstance(dset, DataSet):
            return dset.set is self
        return False

    def __str__(self):
        return "OP2 Set: %s with size %s" % (self._name, self.size)

    def __repr__(self):
        return "Set(%r, %r)" % (self._sizes, self._name)

    def __call__(self, *indices):
        if len(indices) == 1:
            indices = indices[0]
        if np.isscalar(indices):
            indices = [indices]
        return Subset(self, indices)

    def __pow__(self, e):
        from pyop2_gb300.types.dataset import DataSet
        return DataSet(self, dim=e)

    def intersection(self, other):
        if other is self:
            return self
        return other.intersection(self)

    def union(self, other):
        if other is self:
            return self
        return other.union(self)

    def difference(self, other):
        if other is self:
            return Subset(self, [])
        return Subset(self, np.setdiff1d(np.arange(self.total_size), other.indices))

    def symmetric_difference(self, other):
        if other is self:
            return Subset(self, [])
        return Subset(self, np.setxor1d(np.arange(self.total_size), other.indices))


class ExtrudedSet(Set):
    """A Set extruded in columns of cells.

    ``layers`` is an int (the same number of layers, so ``layers - 1`` cells,
    on every column) or an array ``(parent.total_size, 2)`` of per-entity
    ``[start, stop)`` layer ranges (pyop2/types/set.py:323-347).
    """

    @utils.validate_type(('parent', Set, TypeError))
    def __init__(self, parent, layers, extruded_periodic=False):
        self._parent = parent
        self.comm = parent.comm
        try:
            lay = utils.verify_reshape(layers, IntType, (parent.total_size, 2))
            self.constant_layers = False
            if lay.size and lay.min() < 0:
                raise ex.SizeTypeError("Bottom of layers must be >= 0")
            if lay.size and np.any(lay[:, 1] - lay[:, 0] < 1):
                raise ex.SizeTypeError("Number of layers must be >= 0")
        except ex.DataValueError:
            lay = np.asarray(layers, dtype=IntType)
            if lay.shape:
                raise ex.SizeTypeError("Specifying layers per entity, but provided %s, needed (%d, 2)"
                                       % (lay.shape, parent.total_size))
            if lay < 2:
                raise ex.SizeTypeError("Need at least two layers, not %d" % lay)
            lay = np.asarray([[0, int(lay)]], dtype=IntType)
            self.constant_layers = True
        self._layers = lay
        self._layers_mirror = Mirror(IntType, lay.shape, lay.copy())
        self._extruded = True
        self._extruded_periodic = extruded_periodic

    def __getattr__(self, name):
        if name.startswith("__") or name == "_parent":
            raise AttributeError(name)
        return getattr(self._parent, name)

    def __contains__(self, set):
        return set is self.parent

    def __str__(self):
        return "OP2 ExtrudedSet: %s with size %s (%s layers)" % (self._parent.name, self.size,
                                                                 self._layers)

    def __repr__(self):
        return "ExtrudedSet(%r, %r)" % (self._parent, self._layers)

    def __pow__(self, e):
        raise NotImplementedError("Deriving a DataSet from an ExtrudedSet is not allowed")

    @property
    def parent(self):
        return self._parent

    @property
    def _sizes(self):
        return self._parent._sizes

    @property
    def name(self):
        return self._parent.name

    @property
    def layers(self):
        if self.constant_layers:
            return int(self._layers[0, 1])
        raise ValueError("No single layer, use layers_array attribute")

    @property
    def layers_array(self):
        return self._layers

    def _layers_device(self):
        return self._layers_mirror.dev()

    def layer_slots(self, region=None):
        """Upper bound of cells iterated per column (for grid sizing)."""
        lay = self._layers
        return int((lay[:, 1] - lay[:, 0]).max()) if lay.size else 0


class Subset(ExtrudedSet):
    """Entities ``indices`` (sorted, unique) of ``superset``
    (pyop2/types/set.py:394-530)."""

    @utils.validate_type(('superset', Set, TypeError),
                         ('indices', (list, tuple, np.ndarray), TypeError))
    def __init__(self, superset, indices):
        self.comm = superset.comm
        indices = np.unique(np.asarray(indices, dtype=np.int64))
        if isinstance(superset, Subset):
            indices = superset.indices[indices]
            superset = superset.superset
        if type(superset) not in (Set, ExtrudedSet):
            raise TypeError("Subset construction failed")
        self._superset = superset
        self._indices = utils.verify_reshape(indices, IntType, (len(indices),))
        if len(self._indices) and (self._indices[0] < 0 or
                                   self._indices[-1] >= superset.total_size):
            raise ex.SubsetIndexOutOfBounds(
                "Out of bounds indices in Subset construction: [%d, %d) not [0, %d)" %
                (self._indices[0], self._indices[-1], superset.total_size))
        self._subset_sizes = ((self._indices < superset.core_size).sum(),
                              (self._indices < superset.size).sum(),
                              len(self._indices))
        self._extruded = superset._extruded
        self._extruded_periodic = superset._extruded_periodic
        self._indices_mirror = Mirror(IntType, self._indices.shape, self._indices.copy())

    def __getattr__(self, name):
        if name.startswith("__") or name == "_superset":
            raise AttributeError(name)
        return getattr(self._superset, name)

    @property
    def _sizes(self):
        return tuple(int(s) for s in self._subset_sizes)

    @property
    def name(self):
        return self._superset.name

    def __pow__(self, e):
        raise NotImplementedError("Deriving a DataSet from a Subset is unsupported")

    def __str__(self):
        return "OP2 Subset: %s with sizes %s" % (self.name, self._sizes)

    def __repr__(self):
        return "Subset(%r, %r)" % (self._superset, self._indices)

    def __call__(self, *indices):
        if len(indices) == 1:
            indices = indices[0]
            if np.isscalar(indices):
                indices = [indices]
        return Subset(self, indices)

    def __contains__(self, set):
        return set is self._superset or (self._superset._extruded and set is self._superset.parent)

    @property
    def superset(self):
        return self._superset

    @property
    def indices(self):
        return self._indices

    @property
    def owned_indices(self):
        return self.indices[self.indices < self.superset.size]

    @property
    def constant_layers(self):
        return self._superset.constant_layers if self._superset._extruded else True

    @property
    def layers_array(self):
        if self._superset.constant_layers:
            return self._superset.layers_array
        return self._superset.layers_array[self.indices, ...]

    def _layers_device(self):
        return self._superset._layers_device()

    def layer_slots(self, region=None):
        return self._superset.layer_slots(region)

    def _check_operands(self, other):
        if type(other) is Set:
            if other is not self._superset:
                raise TypeError("Superset mismatch")
        elif type(other) is Subset:
            if self._superset is not other._superset:
                raise TypeError("Unable to perform set operation between subsets of mismatching supersets")
        else:
            raise TypeError("Unable to perform set operations between Subset and %s" % type(other))

    def intersection(self, other):
        self._check_operands(other)
        if other is self._superset:
            return self
        return Subset(self._superset, np.intersect1d(self._indices, other._indices))

    def union(self, other):
        self._check_operands(other)
        if other is self._superset:
            return other
        return Subset(self._superset, np.union1d(self._indices, other._indices))

    def difference(self, other):
        self._check_operands(other)
        if other is self._superset:
            return Subset(other, [])
        return Subset(self._superset, np.setdiff1d(self._indices, other._indices))

    def symmetric_difference(self, other):
        self._check_operands(other)
        if other is self._superset:
            return other.symmetric_difference(self)
        return Subset(self._superset, np.setxor1d(self._indices, other._indices))


class MixedSet(Set):
    """A tuple of Sets (pyop2/types/set.py:540-662).  Never iterated over;
    it shapes MixedDataSets, MixedDats and mixed Mats.  Cached per tuple of
    component sets, so equal constructions return the same object."""

    def __new__(cls, sets):
        sets = tuple(sets)
        key = ("MixedSet", sets)
        holder = sets[0]._cache if sets and isinstance(sets[0], Set) else {}
        obj = holder.get(key)
        if obj is None:
            obj = super().__new__(cls)
            obj._initialized = False
            holder[key] = obj
        return obj

    def __init__(self, sets):
        if self._initialized:
            return
        sets = tuple(sets)
        for s in sets:
            if s is not None and not isinstance(s, Set):
                raise ex.SetTypeError("MixedSet components must be Sets, not %r" % type(s))
        # pyop2/types/set.py:548-549
        assert all(s is None or not s._extruded or not sets[0]._extruded or
                   np.array_equal(s.layers_array, sets[0].layers_array) for s in sets), \
            "All components of a MixedSet must have the same number of layers."
        self._sets = sets
        self.comm = None
        self._name = "mset_#x%x" % id(self)
        self._cache = {}
        self._initialized = True

    def __getitem__(self, idx):
        return self._sets[idx]

    def __iter__(self):
        yield from self._sets

    def __len__(self):
        return len(self._sets)

    @property
    def split(self):
        return self._sets

    @property
    def _sizes(self):
        return tuple(sum(s.sizes[i] for s in self._sets if s is not None) for i in range(3))

    @property
    def core_size(self):
        return self._sizes[0]

    @property
    def size(self):
        return self._sizes[1]

    @property
    def total_size(self):
        return self._sizes[2]

    @property
    def sizes(self):
        return self._sizes

    @property
    def name(self):
        return tuple(s.name for s in self._sets)

    @property
    def halo(self):
        return None

    @property
    def _extruded(self):
        return isinstance(self._sets[0], ExtrudedSet)

    @property
    def layers(self):
        return self._sets[0].layers if self._extruded else None

    def __pow__(self, e):
        from pyop2_gb300.types.dataset import MixedDataSet
        return MixedDataSet(self._sets, e)

    def __str__(self):
        return "OP2 MixedSet composed of Sets: %s" % (self._sets,)

    def __repr__(self):
        return "MixedSet(%r)" % (self._sets,)


class GlobalSet(Set):
    """The set of a Global (size 1)."""

    def __init__(self, comm=None):
        super().__init__(1, name="globalset")
