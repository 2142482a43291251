"""The reference's non-legacy loop interface (pyop2/global_kernel.py:19-340):
kernel-argument descriptors and GlobalKernel, the description a Parloop is
built from.

Here a GlobalKernel compiles nothing: the CUDA wrapper is generated, compiled
and cached from the loop's concrete arguments when the Parloop first runs.
What a GlobalKernel needs is a key that identifies the wrapper it describes,
and that key is built from the same tables libop2g is given
(``op2g_map_desc`` / ``op2g_arg_desc``, include/op2g.h): the map descriptors
are flattened into a table of plain, permuted and composed entries, numbered
in order of first appearance (by descriptor identity, so two arguments
through one map share an entry), and each argument becomes a row naming its
kind, shape and the table entries it reads through.

The class names, constructor fields, properties and error messages are the
reference's public interface and stay as user code expects them.
"""
import collections.abc
from typing import Any, Optional, Tuple

from pyop2_gb300.types.access import Access
from pyop2_gb300.types.glob import Constant


class _Frozen:
    """Immutable record: fields are set once by the constructor."""

    __slots__ = ()

    def __setattr__(self, name, value):
        raise AttributeError("%s is immutable" % type(self).__name__)

    def _set(self, **fields):
        for k, v in fields.items():
            object.__setattr__(self, k, v)

    def __repr__(self):
        body = ", ".join("%s=%r" % (k, getattr(self, k)) for k in self.__slots__)
        return "%s(%s)" % (type(self).__name__, body)


def _hashable(value, what):
    if not isinstance(value, collections.abc.Hashable):
        raise ValueError("The provided %s must be hashable" % what)
    return value


# ------------------------------------------------------------ map descriptors
# Map descriptors compare by identity: which arguments share a map is part of
# the loop's signature.
class MapKernelArg(_Frozen):
    """Arity and extruded offsets of a plain map (pyop2/global_kernel.py:19-37)."""

    __slots__ = ("arity", "offset", "offset_quotient")

    def __init__(self, arity: int, offset: Optional[Tuple[int, ...]] = None,
                 offset_quotient: Optional[Tuple[int, ...]] = None):
        self._set(arity=arity, offset=_hashable(offset, "offset"),
                  offset_quotient=_hashable(offset_quotient, "offset_quotient"))

    @property
    def cache_key(self):
        return ("plain", self.arity, self.offset, self.offset_quotient)


class PermutedMapKernelArg(_Frozen):
    """A plain map read through a permutation of its columns
    (pyop2/global_kernel.py:40-53)."""

    __slots__ = ("base_map", "permutation")

    def __init__(self, base_map: MapKernelArg, permutation: Tuple[int, ...]):
        self._set(base_map=base_map, permutation=_hashable(permutation, "permutation"))

    @property
    def cache_key(self):
        return ("permuted", self.base_map.cache_key, tuple(self.permutation))


class ComposedMapKernelArg(_Frozen):
    """A chain of maps, outermost first (pyop2/global_kernel.py:56-74)."""

    __slots__ = ("base_maps",)

    def __init__(self, *base_maps):
        if not all(isinstance(m, _MAP_DESCS) for m in base_maps):
            raise TypeError("base_maps must be a combination of MapKernelArgs, "
                            "PermutedMapKernelArgs, and ComposedMapKernelArgs")
        self._set(base_maps=tuple(base_maps))

    @property
    def cache_key(self):
        return ("composed",) + tuple(m.cache_key for m in self.base_maps)


_MAP_DESCS = (MapKernelArg, PermutedMapKernelArg, ComposedMapKernelArg)


# ------------------------------------------------------- argument descriptors
# These compare by value (two Dat arguments of one shape through one map
# descriptor are the same argument).
class _ValueDesc(_Frozen):
    __slots__ = ()

    def _fields(self):
        return tuple(getattr(self, k) for k in self.__slots__)

    def __eq__(self, other):
        return type(other) is type(self) and other._fields() == self._fields()

    def __hash__(self):
        return hash((type(self).__name__,) + self._fields())

    @property
    def maps(self):
        return ()


class GlobalKernelArg(_ValueDesc):
    """An op2.Global argument of shape ``dim`` (pyop2/global_kernel.py:77-88)."""

    __slots__ = ("dim",)

    def __init__(self, dim: Tuple[int, ...]):
        self._set(dim=dim)

    @property
    def cache_key(self):
        return ("global", self.dim)


class DatKernelArg(_ValueDesc):
    """An op2.Dat argument: per-entity shape ``dim``, the map it is read
    through (None: direct), and for a DatView the component ``index``
    (pyop2/global_kernel.py:91-125)."""

    __slots__ = ("dim", "map_", "index")

    def __init__(self, dim: Tuple[int, ...], map_: Any = None,
                 index: Optional[Tuple[int, ...]] = None):
        self._set(dim=dim, map_=map_, index=index)

    @property
    def is_direct(self):
        return self.map_ is None

    @property
    def is_indirect(self):
        return self.map_ is not None

    @property
    def cache_key(self):
        return ("dat", self.dim, None if self.map_ is None else self.map_.cache_key, self.index)

    @property
    def maps(self):
        return () if self.map_ is None else (self.map_,)


class MatKernelArg(_ValueDesc):
    """An op2.Mat argument: block shapes and (row, column) map descriptors
    (pyop2/global_kernel.py:128-152)."""

    __slots__ = ("dims", "maps", "unroll")

    def __init__(self, dims, maps, unroll: bool = False):
        self._set(dims=dims, maps=tuple(maps), unroll=unroll)

    @property
    def cache_key(self):
        return ("mat", self.dims, tuple(m.cache_key for m in self.maps), self.unroll)


class _MixedDesc(_ValueDesc):
    __slots__ = ()

    def __iter__(self):
        return iter(self.arguments)

    def __len__(self):
        return len(self.arguments)

    @property
    def maps(self):
        return tuple(m for a in self.arguments for m in a.maps)


class MixedDatKernelArg(_MixedDesc):
    """The components of a MixedDat, one kernel parameter
    (pyop2/global_kernel.py:155-175)."""

    __slots__ = ("arguments",)

    def __init__(self, arguments: Tuple[DatKernelArg, ...]):
        self._set(arguments=tuple(arguments))

    @property
    def cache_key(self):
        return ("mixed dat",) + tuple(a.cache_key for a in self.arguments)


class MixedMatKernelArg(_MixedDesc):
    """The blocks of a mixed Mat in row-major block order, block grid
    ``shape`` (pyop2/global_kernel.py:178-206)."""

    __slots__ = ("arguments", "shape")

    def __init__(self, arguments: Tuple[MatKernelArg, ...], shape: Tuple[int, ...]):
        self._set(arguments=tuple(arguments), shape=shape)

    @property
    def cache_key(self):
        return ("mixed mat", self.shape) + tuple(a.cache_key for a in self.arguments)


class PassthroughKernelArg(_ValueDesc):
    """A raw pointer handed to the kernel (pyop2/global_kernel.py:209-219)."""

    __slots__ = ()

    @property
    def cache_key(self):
        return ("passthrough",)


# ---------------------------------------------------------- signature tables
class _DescTable:
    """Map descriptors in the form of libop2g's map table: one entry per
    distinct descriptor object, in order of first appearance; permuted
    entries point at their base map's entry, composed ones list the entries
    of their chain (innermost maps first registered, as the wrapper reads
    them)."""

    def __init__(self):
        self.entries = []
        self._index = {}

    def add(self, m):
        hit = self._index.get(id(m))
        if hit is not None:
            return hit
        if isinstance(m, ComposedMapKernelArg):
            entry = ("composed", tuple(self.add(c) for c in m.base_maps))
        elif isinstance(m, PermutedMapKernelArg):
            entry = ("permuted", self.add(m.base_map), tuple(m.permutation))
        elif isinstance(m, MapKernelArg):
            entry = ("plain", m.arity, m.offset, m.offset_quotient)
        else:
            raise TypeError("not a map descriptor: %r" % (m,))
        # the descriptors are alive while the table is built, so their ids
        # are unique for its lifetime
        self._index[id(m)] = len(self.entries)
        self.entries.append(entry)
        return self._index[id(m)]


def _arg_rows(arguments, table):
    """One row per kernel parameter: its kind and shape, with maps replaced
    by their table entries."""
    rows = []
    for a in arguments:
        if isinstance(a, DatKernelArg):
            rows.append(("dat", a.dim, -1 if a.map_ is None else table.add(a.map_), a.index))
        elif isinstance(a, MatKernelArg):
            rows.append(("mat", a.dims, tuple(table.add(m) for m in a.maps), a.unroll))
        elif isinstance(a, _MixedDesc):
            rows.append((type(a).__name__, getattr(a, "shape", None),
                         tuple(_arg_rows(a.arguments, table))))
        elif isinstance(a, (GlobalKernelArg, PassthroughKernelArg)):
            rows.append(a.cache_key)
        else:
            raise TypeError("not a kernel argument descriptor: %r" % (a,))
    return rows


class GlobalKernel:
    """``GlobalKernel(local_kernel, arguments, *, extruded=False,
    extruded_periodic=False, constant_layers=False, subset=False,
    iteration_region=None, pass_layer_arg=False)`` (pyop2/global_kernel.py:
    248-320): the description of one generated wrapper."""

    def __init__(self, local_kernel, arguments, *, extruded=False, extruded_periodic=False,
                 constant_layers=False, subset=False, iteration_region=None,
                 pass_layer_arg=False):
        if local_kernel.accesses is None or len(local_kernel.accesses) != len(arguments):
            raise ValueError("Number of arguments passed to the local and global kernels"
                             " do not match")
        if pass_layer_arg and not extruded:
            raise ValueError("Cannot request layer argument for non-extruded iteration")
        if constant_layers and not extruded:
            raise ValueError("Cannot request constant_layers argument for non-extruded "
                             "iteration")
        self.local_kernel = local_kernel
        self.arguments = tuple(arguments)
        self._extruded = extruded
        self._extruded_periodic = extruded_periodic
        self._constant_layers = constant_layers
        self._subset = subset
        self._iteration_region = iteration_region
        self._pass_layer_arg = pass_layer_arg
        table = _DescTable()
        rows = tuple(_arg_rows(self.arguments, table))
        flags = (("extruded", extruded), ("extruded_periodic", extruded_periodic),
                 ("constant_layers", constant_layers), ("subset", subset),
                 ("iteration_region", iteration_region), ("pass_layer_arg", pass_layer_arg))
        self.cache_key = (local_kernel.cache_key, rows, tuple(table.entries), flags)

    @property
    def name(self):
        return "wrap_%s" % self.local_kernel.name

    @property
    def num_flops(self):
        return self.local_kernel.flop_count or 0


def check_constants(global_knl, arguments):
    """A Constant may only be read (pyop2/global_kernel.py:287-294)."""
    for acc, parg in zip(global_knl.local_kernel.accesses, arguments):
        if isinstance(getattr(parg, "data", None), Constant) and acc is not Access.READ:
            raise ValueError("Constants can only ever be read in a parloop, not modified")
