"""The reference's non-legacy loop interface (pyop2/global_kernel.py:19-340):
kernel-argument descriptors and GlobalKernel, the signature a Parloop is
built from.  Here a GlobalKernel is only a description: the generated CUDA
wrapper is compiled (and cached) from the concrete arguments when the
Parloop first runs."""
import collections.abc
import itertools
from dataclasses import dataclass
from typing import Optional, Tuple

from pyop2_gb300.types.access import Access
from pyop2_gb300.types.glob import Constant


@dataclass(eq=False, frozen=True)
class MapKernelArg:
    """A map argument: arity and extruded offsets (pyop2/global_kernel.py:19-37)."""
    arity: int
    offset: Optional[Tuple[int, ...]] = None
    offset_quotient: Optional[Tuple[int, ...]] = None

    def __post_init__(self):
        if not isinstance(self.offset, collections.abc.Hashable):
            raise ValueError("The provided offset must be hashable")
        if not isinstance(self.offset_quotient, collections.abc.Hashable):
            raise ValueError("The provided offset_quotient must be hashable")

    @property
    def cache_key(self):
        return type(self), self.arity, self.offset, self.offset_quotient


@dataclass(eq=False, frozen=True)
class PermutedMapKernelArg:
    base_map: MapKernelArg
    permutation: Tuple[int, ...]

    def __post_init__(self):
        if not isinstance(self.permutation, collections.abc.Hashable):
            raise ValueError("The provided permutation must be hashable")

    @property
    def cache_key(self):
        return type(self), self.base_map.cache_key, tuple(self.permutation)


class ComposedMapKernelArg:
    def __init__(self, *base_maps):
        for m in base_maps:
            if not isinstance(m, (MapKernelArg, PermutedMapKernelArg, ComposedMapKernelArg)):
                raise TypeError("base_maps must be a combination of MapKernelArgs, "
                                "PermutedMapKernelArgs, and ComposedMapKernelArgs")
        self.base_maps = base_maps

    @property
    def cache_key(self):
        return type(self), tuple(m.cache_key for m in self.base_maps)


@dataclass(frozen=True)
class GlobalKernelArg:
    dim: Tuple[int, ...]

    @property
    def cache_key(self):
        return type(self), self.dim

    @property
    def maps(self):
        return ()


@dataclass(frozen=True)
class DatKernelArg:
    dim: Tuple[int, ...]
    map_: object = None
    index: Optional[Tuple[int, ...]] = None

    @property
    def is_direct(self):
        return self.map_ is None

    @property
    def is_indirect(self):
        return not self.is_direct

    @property
    def cache_key(self):
        return type(self), self.dim, self.map_.cache_key if self.map_ is not None else None, \
            self.index

    @property
    def maps(self):
        return (self.map_,) if self.map_ is not None else ()


@dataclass(frozen=True)
class MatKernelArg:
    dims: Tuple[Tuple[int, ...], Tuple[int, ...]]
    maps: Tuple[MapKernelArg, MapKernelArg]
    unroll: bool = False

    @property
    def cache_key(self):
        return type(self), self.dims, tuple(m.cache_key for m in self.maps), self.unroll


@dataclass(frozen=True)
class MixedDatKernelArg:
    arguments: Tuple[DatKernelArg, ...]

    def __iter__(self):
        return iter(self.arguments)

    def __len__(self):
        return len(self.arguments)

    @property
    def cache_key(self):
        return tuple(a.cache_key for a in self.arguments)

    @property
    def maps(self):
        return tuple(m for a in self.arguments for m in a.maps)


@dataclass(frozen=True)
class MixedMatKernelArg:
    arguments: Tuple[MatKernelArg, ...]
    shape: Tuple[int, ...]

    def __iter__(self):
        return iter(self.arguments)

    def __len__(self):
        return len(self.arguments)

    @property
    def cache_key(self):
        return tuple(a.cache_key for a in self.arguments)

    @property
    def maps(self):
        return tuple(m for a in self.arguments for m in a.maps)


class PassthroughKernelArg:
    @property
    def cache_key(self):
        return type(self)

    @property
    def maps(self):
        return ()


class GlobalKernel:
    """``GlobalKernel(local_kernel, arguments, *, extruded=False,
    extruded_periodic=False, constant_layers=False, subset=False,
    iteration_region=None, pass_layer_arg=False)`` (pyop2/global_kernel.py:
    248-320): validates the description and keys it as the reference does."""

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
        counter = itertools.count()
        seen_maps = collections.defaultdict(lambda: next(counter))
        self.cache_key = (local_kernel.cache_key, *[a.cache_key for a in arguments],
                          *[seen_maps[m] for a in arguments for m in a.maps],
                          extruded, extruded_periodic, constant_layers, subset,
                          iteration_region, pass_layer_arg)
        self.local_kernel = local_kernel
        self.arguments = tuple(arguments)
        self._extruded = extruded
        self._extruded_periodic = extruded_periodic
        self._constant_layers = constant_layers
        self._subset = subset
        self._iteration_region = iteration_region
        self._pass_layer_arg = pass_layer_arg

    @property
    def name(self):
        return "wrap_%s" % self.local_kernel.name

    @property
    def num_flops(self):
        return self.local_kernel.flop_count or 0


def check_constants(global_knl, arguments):
    """Constants may only be READ (pyop2/global_kernel.py:287-294)."""
    for acc, parg in zip(global_knl.local_kernel.accesses, arguments):
        if isinstance(getattr(parg, "data", None), Constant) and acc is not Access.READ:
            raise ValueError("Constants can only ever be read in a parloop, not modified")
