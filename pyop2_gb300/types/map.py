"""Maps (pyop2/types/map.py): Map :17-168, PermutedMap :171-215,
ComposedMap :218-294, MixedMap :297-434.

Map values live on the device as int32 ``[iterset.total_size, arity]``; the
host copy is kept read-only so the two can never diverge.
"""
import itertools
import numbers

import numpy as np

from pyop2_gb300 import exceptions as ex
from pyop2_gb300 import utils
from pyop2_gb300.datatypes import IntType
from pyop2_gb300.device import Mirror
from pyop2_gb300.types.set import Set


class Map:
    """Each entity of ``iterset`` maps to ``arity`` entities of ``toset``.

    ``offset`` (length arity) is the per-layer increment of the values for
    extruded iteration; ``offset_quotient`` is used by periodic extrusion.
    """

    dtype = IntType
    # Serial numbers: unlike id(), never reused within a process, so caches
    # keyed by them (colouring plans) cannot hand one map's result to another.
    _serials = itertools.count()

    @utils.validate_type(('iterset', Set, ex.SetTypeError), ('toset', Set, ex.SetTypeError),
                         ('arity', numbers.Integral, ex.ArityTypeError),
                         ('name', str, ex.NameTypeError))
    def __init__(self, iterset, toset, arity, values=None, name=None, offset=None,
                 offset_quotient=None):
        self._iterset = iterset
        self._toset = toset
        self.comm = toset.comm
        self._arity = int(arity)
        self._values = utils.verify_reshape(values, IntType, (iterset.total_size, arity),
                                            allow_none=True)
        self.shape = (iterset.total_size, arity)
        self._name = name or "map_#x%x" % id(self)
        if offset is None or len(offset) == 0:
            self._offset = None
        else:
            self._offset = utils.verify_reshape(offset, IntType, (arity,))
        if offset_quotient is None or len(offset_quotient) == 0:
            self._offset_quotient = None
        else:
            self._offset_quotient = utils.verify_reshape(offset_quotient, IntType, (arity,))
        self._cache = {}
        self._mirror = None

    @property
    def _serial(self):
        """This map's serial number, drawn at first use (every Map kind)."""
        s = self.__dict__.get("_serial_no")
        if s is None:
            s = self.__dict__["_serial_no"] = next(Map._serials)
        return s

    # ---- device
    def _device_values(self):
        """Device int32 buffer of the values, uploaded at first use; from then
        on the host array is read-only, so the two copies cannot diverge."""
        if self._mirror is None:
            self._values.setflags(write=False)
            self._mirror = Mirror(IntType, self._values.shape, self._values)
            dev = self._mirror.dev()
            from pyop2_gb300.configuration import configuration
            if configuration["check_maps"] and not configuration["debug"]:
                self._check_bounds(dev)
        return self._mirror.dev()

    def _check_bounds(self, dev):
        """Refuse values that would index outside the target set.  The
        reference does not check (it would read or write past the array on
        the CPU); on the GPU such an access faults the context, so the values
        of every entity are checked once, on the device, when they
        are uploaded: every non-negative value (negative ones are skipped by
        the wrappers), plus its layer offset times the largest layer term
        an extruded loop forms (cell layers - 1 for every iteration region),
        must be below ``toset.total_size``."""
        import torch
        n, a = self._iterset.total_size, self._arity     # ghost rows too: a Subset may use them
        if n == 0 or a == 0:
            return
        v = dev[:self._values.nbytes].view(torch.int32).view(n, a)
        v = v.to(torch.int64)
        hi = v
        it = self._iterset
        if getattr(it, "_extruded", False) and self._offset is not None:
            lay = np.asarray(it.layers_array, dtype=np.int64).reshape(-1, 2)
            terms = lay[:, 1] - lay[:, 0] - 2          # cell layers - 1
            if len(terms) == 1:
                terms = np.full(n, terms[0])
            else:
                terms = terms[:n]
            terms = np.maximum(terms, 0)
            off = np.maximum(np.asarray(self._offset, dtype=np.int64), 0)
            hi = v + torch.as_tensor(terms[:, None] * off[None, :], device=v.device)
        hi = torch.where(v >= 0, hi, torch.zeros_like(hi))
        m = int(hi.max().item())
        if m >= self._toset.total_size:
            raise ex.MapValueError("Map %s: entry %d (with its layer offset) is outside the "
                                   "target set %s of size %d" % (self._name, m, self._toset.name,
                                                                 self._toset.total_size))

    @property
    def _global_kernel_arg(self):
        """This map's descriptor, one object per map (arguments through the
        same map share it, which is how a GlobalKernel's key sees the map
        shared)."""
        d = self.__dict__.get("_gk_arg")
        if d is None:
            from pyop2_gb300.global_kernel import MapKernelArg
            d = self.__dict__["_gk_arg"] = MapKernelArg(
                self.arity, utils.tuplify(self.offset), utils.tuplify(self.offset_quotient))
        return d

    @property
    def _cache_key(self):
        """What of this map determines generated code (pyop2/types/map.py:60-62)."""
        return (type(self).__name__, self.arity, utils.tuplify(self.offset),
                utils.tuplify(self.offset_quotient))

    def __iter__(self):
        yield self

    def __len__(self):
        return 1

    @property
    def split(self):
        return (self,)

    @property
    def iterset(self):
        return self._iterset

    @property
    def toset(self):
        return self._toset

    @property
    def arity(self):
        return self._arity

    @property
    def arities(self):
        return (self._arity,)

    @property
    def arange(self):
        return (0, self._arity)

    @property
    def values(self):
        return self._values[:self.iterset.size]

    @property
    def values_with_halo(self):
        return self._values

    @property
    def name(self):
        return self._name

    @property
    def offset(self):
        return self._offset

    @property
    def offset_quotient(self):
        return self._offset_quotient

    @property
    def flattened_maps(self):
        return (self,)

    def __str__(self):
        return "OP2 Map: %s from (%s) to (%s) with arity %s" % (self._name, self._iterset,
                                                               self._toset, self._arity)

    def __repr__(self):
        return "Map(%r, %r, %r, None, %r, %r, %r)" % (self._iterset, self._toset, self._arity,
                                                    self._name, self._offset,
                                                    self._offset_quotient)

    def __le__(self, o):
        return self == o


class PermutedMap(Map):
    """``local[i] = global[map[permutation[i]]]`` (pyop2/types/map.py:171-215)."""

    @property
    def _global_kernel_arg(self):
        d = self.__dict__.get("_gk_arg")
        if d is None:
            from pyop2_gb300.global_kernel import PermutedMapKernelArg
            d = self.__dict__["_gk_arg"] = PermutedMapKernelArg(self.map_._global_kernel_arg,
                                                                tuple(self.permutation))
        return d

    def __init__(self, map_, permutation):
        if not isinstance(map_, Map):
            raise TypeError("map_ must be a Map instance")
        if isinstance(map_, ComposedMap):
            raise NotImplementedError("PermutedMap of ComposedMap not implemented: simply "
                                      "permute before composing")
        self.map_ = map_
        self.comm = map_.comm
        self.permutation = np.asarray(permutation, dtype=IntType)
        assert (np.unique(self.permutation) == np.arange(map_.arity, dtype=IntType)).all()

    @property
    def _cache_key(self):
        return self.map_._cache_key + (tuple(self.permutation),)

    def __getattr__(self, name):
        if name.startswith("__") or name == "map_":
            raise AttributeError(name)
        return getattr(self.map_, name)

    @property
    def iterset(self):
        return self.map_.iterset

    @property
    def toset(self):
        return self.map_.toset

    @property
    def arity(self):
        return self.map_.arity

    @property
    def offset(self):
        return self.map_.offset

    @property
    def offset_quotient(self):
        return self.map_.offset_quotient

    @property
    def values_with_halo(self):
        return self.map_.values_with_halo

    @property
    def values(self):
        return self.map_.values

    @property
    def flattened_maps(self):
        return (self,)


class ComposedMap(Map):
    """``local[i] = global[maps_[0][maps_[1][...[n]]][i]]``; inner maps have
    arity 1 (pyop2/types/map.py:218-294)."""

    @property
    def _global_kernel_arg(self):
        d = self.__dict__.get("_gk_arg")
        if d is None:
            from pyop2_gb300.global_kernel import ComposedMapKernelArg
            d = self.__dict__["_gk_arg"] = ComposedMapKernelArg(
                *(m._global_kernel_arg for m in self.maps_))
        return d

    def __init__(self, *maps_, name=None):
        if not all(isinstance(m, Map) for m in maps_):
            raise TypeError("All maps must be Map instances")
        for tomap, frommap in zip(maps_[:-1], maps_[1:]):
            if tomap.iterset is not frommap.toset:
                raise ex.MapTypeError("tomap.iterset must match frommap.toset")
            if frommap.arity != 1:
                raise ex.MapTypeError("frommap.arity must be 1")
        self._iterset = maps_[-1].iterset
        self._toset = maps_[0].toset
        self.comm = self._toset.comm
        self._arity = maps_[0].arity
        self._values = None
        self.shape = (self._iterset.total_size, self._arity)
        self._name = name or "cmap_#x%x" % id(self)
        self._offset = maps_[0].offset
        self._offset_quotient = maps_[0].offset_quotient
        self._cache = {}
        self.maps_ = tuple(maps_)

    @property
    def _cache_key(self):
        return tuple(m._cache_key for m in self.maps_)

    @property
    def values(self):
        raise RuntimeError("ComposedMap does not store values directly")

    @property
    def values_with_halo(self):
        raise RuntimeError("ComposedMap does not store values directly")

    def __str__(self):
        return "OP2 ComposedMap of Maps: [%s]" % ",".join(str(m) for m in self.maps_)

    def __repr__(self):
        return "ComposedMap(%s)" % ",".join(repr(m) for m in self.maps_)

    def __le__(self, o):
        raise NotImplementedError("__le__ not implemented for ComposedMap")

    @property
    def flattened_maps(self):
        return tuple(itertools.chain(*(m.flattened_maps for m in self.maps_)))


class MixedMap(Map):
    """A tuple of Maps from one iteration set (pyop2/types/map.py:297-434).
    Cached per tuple of component maps.  Used with a MixedDat (one pack
    concatenating the components' packs) or as a mixed Mat's row/column map."""

    def __new__(cls, maps):
        maps = tuple(maps)
        for m in maps:
            if not isinstance(m, Map):
                raise ex.MapTypeError("MixedMap components must be Maps, not %r" % type(m))
        key = ("MixedMap", maps)
        holder = maps[0]._cache
        obj = holder.get(key)
        if obj is None:
            obj = object.__new__(cls)
            obj._initialized = False
            holder[key] = obj
        return obj

    def __init__(self, maps):
        if self._initialized:
            return
        maps = tuple(maps)
        for m in maps:
            if not isinstance(m, Map):
                raise ex.MapTypeError("MixedMap components must be Maps, not %r" % type(m))
        if len(set(id(m.iterset) for m in maps)) != 1:
            raise RuntimeError("Found multiple itersets.")
        self._maps = maps
        self.comm = None
        self._name = "mmap_#x%x" % id(self)
        self._cache = {}
        self._initialized = True

    @property
    def split(self):
        return self._maps

    def __iter__(self):
        yield from self._maps

    def __len__(self):
        return len(self._maps)

    def __getitem__(self, idx):
        return self._maps[idx]

    @property
    def iterset(self):
        return self._maps[0].iterset

    @property
    def toset(self):
        from pyop2_gb300.types.set import MixedSet
        return MixedSet(tuple(m.toset for m in self._maps))

    @property
    def arity(self):
        return sum(m.arity for m in self._maps)

    @property
    def arities(self):
        return tuple(m.arity for m in self._maps)

    @property
    def arange(self):
        return (0,) + tuple(int(x) for x in np.cumsum(self.arities))

    @property
    def values(self):
        return tuple(m.values for m in self._maps)

    @property
    def values_with_halo(self):
        return tuple(m.values_with_halo for m in self._maps)

    @property
    def name(self):
        return tuple(m.name for m in self._maps)

    @property
    def offset(self):
        return tuple(m.offset for m in self._maps)

    @property
    def offset_quotient(self):
        return tuple(m.offset_quotient for m in self._maps)

    @property
    def flattened_maps(self):
        raise NotImplementedError("flattened_maps is not defined for a MixedMap")

    def __le__(self, o):
        return self is o or all(m <= om for m, om in zip(self, o))

    def __str__(self):
        return "OP2 MixedMap composed of Maps: %s" % (self._maps,)

    def __repr__(self):
        return "MixedMap(%r)" % (self._maps,)
