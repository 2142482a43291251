"""par_loop orchestration (pyop2/parloop.py:167-760) on the GPU.

``op2.par_loop(kernel, iterset, *args)`` validates its arguments exactly as
the reference does, builds a descriptor of the loop signature, obtains the
compiled wrapper for that signature from libop2g (generated CUDA around the
user kernel, NVRTC-compiled, cached by signature) and launches it on torch's
current stream.  The loop executes [0, iterset.size) in one launch: on one
GPU there is no halo exchange to overlap, so the reference's core/owned split
(pyop2/parloop.py:243-260) collapses to a single range.

INC/MIN/MAX conflicts through maps are resolved by hardware atomics (default),
warp-aggregated atomics, or a greedy colouring with one launch per colour
(``configuration['scatter']``; ``'auto'`` lets the autotuner choose).
"""
import collections
import ctypes
from dataclasses import dataclass
from typing import Any, Optional, Tuple

import numpy as np
import torch

from pyop2_gb300 import _lib, device
from pyop2_gb300.configuration import configuration
from pyop2_gb300.datatypes import IntType, as_code
from pyop2_gb300.exceptions import KernelTypeError, MapValueError, SetTypeError
from pyop2_gb300.local_kernel import CStringLocalKernel, LocalKernel
from pyop2_gb300.types.access import ALL, Access, IterationRegion
from pyop2_gb300.types.dat import Dat, DatView
from pyop2_gb300.types.glob import Constant, Global
from pyop2_gb300.types.map import ComposedMap, Map, MixedMap, PermutedMap
from pyop2_gb300.types.mat import Mat
from pyop2_gb300.types.set import ExtrudedSet, MixedSet, Set, Subset


# --------------------------------------------------------------- legacy args
class LegacyArg:
    """Old-style par_loop argument: data + access (+ maps)."""


@dataclass
class GlobalLegacyArg(LegacyArg):
    data: Global
    access: Access

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def global_kernel_arg(self):
        from pyop2_gb300.global_kernel import GlobalKernelArg
        return GlobalKernelArg(self.data.dim)

    @property
    def parloop_arg(self):
        return GlobalParloopArg(self.data)

    @property
    def maps(self):
        return ()


@dataclass
class DatLegacyArg(LegacyArg):
    data: Dat
    map_: Optional[Map]
    access: Access

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def global_kernel_arg(self):
        from pyop2_gb300.global_kernel import DatKernelArg
        m = self.map_._global_kernel_arg if self.map_ is not None else None
        index = self.data.index if isinstance(self.data, DatView) else None
        return DatKernelArg(self.data.dataset.dim, m, index=index)

    @property
    def parloop_arg(self):
        return DatParloopArg(self.data, self.map_)

    @property
    def maps(self):
        return (self.map_,) if self.map_ is not None else ()


@dataclass
class MatLegacyArg(LegacyArg):
    data: Mat
    maps: Tuple[Map, Map]
    access: Access
    lgmaps: Optional[Tuple[Any, Any]] = None
    needs_unrolling: Optional[bool] = False

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def global_kernel_arg(self):
        from pyop2_gb300.global_kernel import MatKernelArg
        return MatKernelArg(self.data.dims, tuple(m._global_kernel_arg for m in self.maps),
                            unroll=self.needs_unrolling)

    @property
    def parloop_arg(self):
        return MatParloopArg(self.data, self.maps, self.lgmaps)


@dataclass
class MixedDatLegacyArg(LegacyArg):
    """A MixedDat through a MixedMap (pyop2/parloop.py:600-621): one kernel
    argument whose pack concatenates the components' packs."""
    data: Any
    map_: Any
    access: Access

    @property
    def dtype(self):
        return self.data.dtype

    @property
    def maps(self):
        return tuple(self.map_)

    def components(self):
        return [DatLegacyArg(d, m, self.access) for d, m in zip(self.data, self.map_)]

    @property
    def global_kernel_arg(self):
        from pyop2_gb300.global_kernel import MixedDatKernelArg
        return MixedDatKernelArg(tuple(c.global_kernel_arg for c in self.components()))

    @property
    def parloop_arg(self):
        return MixedDatParloopArg(self.data, self.map_)


@dataclass
class MixedMatLegacyArg(LegacyArg):
    """A mixed Mat through a pair of MixedMaps (pyop2/parloop.py:649-678):
    one element matrix over all blocks, block (i, j) inserted into
    ``mat[i, j]`` through ``(rmap.split[i], cmap.split[j])``."""
    data: Mat
    maps: Tuple[Any, Any]
    access: Access
    lgmaps: Optional[Tuple[Any, Any]] = None
    needs_unrolling: Optional[bool] = False

    @property
    def dtype(self):
        return self.data.dtype

    def components(self):
        rm, cm = self.maps
        nr, nc = self.data.sparsity.shape
        return [MatLegacyArg(self.data[i, j], (rm.split[i], cm.split[j]), self.access)
                for i in range(nr) for j in range(nc)]

    @property
    def global_kernel_arg(self):
        from pyop2_gb300.global_kernel import MixedMatKernelArg
        return MixedMatKernelArg(tuple(c.global_kernel_arg for c in self.components()),
                                 shape=self.data.sparsity.shape)

    @property
    def parloop_arg(self):
        return MixedMatParloopArg(self.data, tuple(self.maps), self.lgmaps)


@dataclass
class PassthroughArg(LegacyArg):
    """A raw device pointer handed to the kernel untouched (dtype for codegen)."""
    dtype: Any
    data: int
    access = Access.RW

    @property
    def maps(self):
        return ()

    @property
    def global_kernel_arg(self):
        from pyop2_gb300.global_kernel import PassthroughKernelArg
        return PassthroughKernelArg()

    @property
    def parloop_arg(self):
        return PassthroughParloopArg(self.data)


# ------------------------------------------- non-legacy loop arguments
# (pyop2/parloop.py:30-164): data (+ maps) without the access, which the
# local kernel's ``accesses`` supply.
class ParloopArg:
    pass


@dataclass
class GlobalParloopArg(ParloopArg):
    data: Global

    @property
    def maps(self):
        return ()


@dataclass
class DatParloopArg(ParloopArg):
    data: Dat
    map_: Optional[Map] = None

    @property
    def maps(self):
        return (self.map_,) if self.map_ is not None else ()


@dataclass
class MixedDatParloopArg(ParloopArg):
    data: Any
    map_: Any

    @property
    def maps(self):
        return (self.map_,)


@dataclass
class MatParloopArg(ParloopArg):
    data: Mat
    maps: Tuple[Map, Map]
    lgmaps: Optional[Any] = None


@dataclass
class MixedMatParloopArg(ParloopArg):
    data: Mat
    maps: Tuple[Any, Any]
    lgmaps: Any = None


@dataclass
class PassthroughParloopArg(ParloopArg):
    data: int

    @property
    def maps(self):
        return ()


def _legacy_from(parg, access, dtype, garg):
    """The legacy argument equivalent to a ParloopArg with its access."""
    if isinstance(parg, GlobalParloopArg):
        return GlobalLegacyArg(parg.data, access)
    if isinstance(parg, DatParloopArg):
        return DatLegacyArg(parg.data, parg.map_, access)
    if isinstance(parg, MixedDatParloopArg):
        return MixedDatLegacyArg(parg.data, parg.map_, access)
    if isinstance(parg, MatParloopArg):
        return MatLegacyArg(parg.data, tuple(parg.maps), access, parg.lgmaps,
                            getattr(garg, "unroll", False))
    if isinstance(parg, MixedMatParloopArg):
        return MixedMatLegacyArg(parg.data, tuple(parg.maps), access, parg.lgmaps)
    if isinstance(parg, PassthroughParloopArg):
        return PassthroughArg(dtype if dtype is not None else np.uint8, parg.data)
    raise ValueError("Unhandled argument type %r" % type(parg))


# ------------------------------------------------------------- validation
def _check_map(m):
    if configuration["type_check"]:
        if isinstance(m, MixedMap):
            for m_ in m.split:
                _check_map(m_)
        elif isinstance(m, ComposedMap):
            for m_ in m.maps_:
                _check_map(m_)
        elif isinstance(m, PermutedMap):
            _check_map(m.map_)
        elif m.iterset.total_size > 0 and len(m.values_with_halo) == 0:
            raise MapValueError("%s is not initialized" % m)


def _check_iterset(iterset, args):
    """pyop2/parloop.py:470-499."""
    if not configuration["type_check"]:
        return
    if not isinstance(iterset, Set):
        raise SetTypeError("Iteration set is of the wrong type")
    if isinstance(iterset, MixedSet):
        raise SetTypeError("Cannot iterate over mixed sets")
    if isinstance(iterset, Subset):
        iterset = iterset.superset
    for i, a in enumerate(args):
        if isinstance(a, DatLegacyArg) and a.map_ is None:
            _iterset = iterset.parent if isinstance(iterset, ExtrudedSet) else iterset
            if a.data.dataset.set != _iterset:
                raise MapValueError("Iterset of direct arg %d does not match parloop iterset" % i)
        for j, m in enumerate(a.maps):
            if m.iterset != iterset and m.iterset not in iterset:
                raise MapValueError("Iterset of arg %d map %d does not match parloop iterset" % (i, j))


# ------------------------------------------------------------ signature
class _MapTable:
    """Unique maps of a loop, in first-seen order (pyop2/parloop.py:204-212),
    flattened into plain / permuted / composed entries for libop2g."""

    def __init__(self):
        self.entries = []     # (kind, arity, base, composed tuple, offset, oq, perm)
        self.objs = []        # plain Map object per entry (None otherwise)
        self._index = {}

    def add(self, m):
        key = id(m)
        if key in self._index:
            return self._index[key]
        if isinstance(m, ComposedMap):
            comps = [self.add(c) for c in m.flattened_maps]
            entry = (_lib.MAP_COMPOSED, m.arity, -1, tuple(comps), None, None, None)
            obj = None
        elif isinstance(m, PermutedMap):
            base = self.add(m.map_)
            entry = (_lib.MAP_PERMUTED, m.arity, base, (), None, None,
                     tuple(int(x) for x in m.permutation))
            obj = None
        else:
            off = None if m.offset is None else tuple(int(x) for x in m.offset)
            oq = None if m.offset_quotient is None else tuple(int(x) for x in m.offset_quotient)
            entry = (_lib.MAP_PLAIN, m.arity, -1, (), off, oq, None)
            obj = m
        idx = len(self.entries)
        self.entries.append(entry)
        self.objs.append(obj)
        self._index[key] = idx
        return idx

    def key(self):
        return tuple(self.entries)


_KERNELS = {}   # signature key -> _Compiled


class _Compiled:
    """A libop2g kernel handle with its ctypes descriptors."""

    def __init__(self, handle, nptrs):
        self.handle = handle
        self.nptrs = nptrs

    def __del__(self):
        try:
            if self.handle:
                _lib.lib().op2g_kernel_destroy(self.handle)
        except Exception:
            pass

    def source(self):
        n = ctypes.c_size_t()
        _lib.call("op2g_kernel_source", self.handle, None, 0, ctypes.byref(n))
        buf = ctypes.create_string_buffer(n.value)
        _lib.call("op2g_kernel_source", self.handle, buf, n.value, ctypes.byref(n))
        return buf.value.decode()


def signature_key(code, name, loop, args, maps, arch=None):
    """What identifies a compiled wrapper: kernel code and name, loop flags,
    argument kinds/access/dtype/dims, map shapes with map identity reduced to
    first-seen order (as pyop2/global_kernel.py:304-312 keys GlobalKernel)."""
    return (code, name, tuple(sorted(loop.items())), tuple(args), tuple(maps), arch)


def compile_signature(code, name, loop, args, maps, arch=None):
    """Compile (or fetch) the wrapper for a signature given as plain tuples:
    loop = dict of LoopDesc fields, args = list of ArgDesc field tuples,
    maps = list of _MapTable entries."""
    key = signature_key(code, name, loop, args, maps, arch)
    c = _KERNELS.get(key)
    if c is not None:
        return c
    L = _lib.LoopDesc(**loop)
    A = (_lib.ArgDesc * max(1, len(args)))()
    for i, a in enumerate(args):
        A[i] = _lib.ArgDesc(*a)
    M = (_lib.MapDesc * max(1, len(maps)))()
    keep = []
    for i, (kind, arity, base, comps, off, oq, perm) in enumerate(maps):
        d = M[i]
        d.kind, d.arity, d.base, d.ncomposed = kind, arity, base, len(comps)
        for k, c in enumerate(comps):
            d.composed[k] = c
        for fld, vals in (("offset", off), ("offset_quotient", oq), ("permutation", perm)):
            if vals is not None:
                arr = (ctypes.c_int32 * len(vals))(*vals)
                keep.append(arr)
                setattr(d, fld, ctypes.cast(arr, ctypes.POINTER(ctypes.c_int32)))
    h = ctypes.c_void_p()
    cache_dir = configuration["cache_dir"]
    _lib.call("op2g_kernel_create", code.encode(), name.encode(), ctypes.byref(L), A, len(args),
              M, len(maps), arch.encode() if arch else None,
              cache_dir.encode() if cache_dir else None, ctypes.byref(h))
    c = _Compiled(h.value, _lib.lib().op2g_kernel_num_ptrs(h.value))
    _KERNELS[key] = c
    return c


# ---------------------------------------------------------------- Parloop
class Parloop:
    """A parallel loop invocation (pyop2/parloop.py:167-537).

    ``Parloop(kernel, iterset, args, iteration_region=None,
    pass_layer_arg=False)``; ``compute()`` (or calling it) executes it.
    """

    def __init__(self, local_knl, iterset, args, iteration_region=None, pass_layer_arg=False):
        from pyop2_gb300.global_kernel import GlobalKernel, check_constants
        self._global_kernel = None
        self._parloop_args = None
        if isinstance(local_knl, GlobalKernel):
            # the non-legacy form Parloop(global_kernel, iterset, parloop_args)
            # (pyop2/parloop.py:167-190)
            g = local_knl
            if len(g.arguments) != len(args):
                raise ValueError("You are trying to pass in a different number of arguments "
                                 "than the kernel is expecting")
            check_constants(g, args)
            dtypes = getattr(g.local_kernel, "dtypes", None) or (None,) * len(args)
            self._global_kernel = g
            self._parloop_args = list(args)
            args = [_legacy_from(pa, acc, dt, ga) for pa, acc, dt, ga in
                    zip(args, g.local_kernel.accesses, dtypes, g.arguments)]
            iteration_region = g._iteration_region
            pass_layer_arg = g._pass_layer_arg
            local_knl = g.local_kernel
        if not isinstance(local_knl, LocalKernel):
            raise KernelTypeError
        if pass_layer_arg and not iterset._extruded:
            raise ValueError("Cannot request layer argument for non-extruded iteration")
        for a in args:
            for m in a.maps:
                _check_map(m)
            if isinstance(a, GlobalLegacyArg) and isinstance(a.data, Constant) \
                    and a.access is not Access.READ:
                raise ValueError("Constants can only ever be read in a parloop, not modified")
        _check_iterset(iterset, args)
        self.local_kernel = local_knl
        self.iterset = iterset
        self.args = tuple(args)
        self.iteration_region = IterationRegion(iteration_region or ALL)
        self.pass_layer_arg = bool(pass_layer_arg)
        self._built = None
        self._plan = None
        self._stage = None
        self._flatten()

    def _flatten(self):
        # Arguments as the wrapper sees them: mixed arguments become their
        # components, tagged with a group id (one kernel parameter per group)
        # and, for Mats, the number of block columns.
        flat = []
        group = 0
        for a in self.args:
            if isinstance(a, (MixedDatLegacyArg, MixedMatLegacyArg)):
                group += 1
                cols = a.data.sparsity.shape[1] if isinstance(a, MixedMatLegacyArg) else 0
                flat += [(c, group, cols) for c in a.components()]
            else:
                flat.append((a, 0, 0))
        self._flat = flat
        self._components = [c for c, _, _ in flat]
        self._written = None
        # pyop2/parloop.py:501-511
        for a in self._components:
            if isinstance(a, DatLegacyArg) and a.data._halo_frozen and \
                    a.data._frozen_access_mode != a.access:
                raise RuntimeError("Dats with frozen halos must always be accessed with the "
                                   "same access mode")

    @property
    def accesses(self):
        return tuple(a.access for a in self.args)

    @property
    def global_kernel(self):
        """The GlobalKernel this loop runs (built from legacy arguments when
        the loop was constructed from them)."""
        if self._global_kernel is None:
            self.local_kernel.accesses = self.accesses
            self._global_kernel = global_kernel_of(self.local_kernel, self.iterset, self.args,
                                                   self.iteration_region, self.pass_layer_arg)
        return self._global_kernel

    def replace_data(self, index, new_argument):
        """Run the loop on other data (pyop2/parloop.py:218-219): argument
        ``index`` now refers to ``new_argument``.  The compiled wrapper is
        kept when the signature is unchanged."""
        old_key = self.cache_key()
        a = self.args[index]
        a.data = new_argument
        if self._parloop_args is not None:
            self._parloop_args[index].data = new_argument
        self._flatten()
        self._launch_cache = None
        self._plan = None
        self._stage = None
        if self.cache_key() != old_key:
            self._built = None

    @property
    def arguments(self):
        return tuple(self._parloop_args) if self._parloop_args is not None else self.args

    # ---- signature
    def _signature(self):
        table = _MapTable()
        argdescs = []
        for a, group, gcols in self._flat:
            if isinstance(a, GlobalLegacyArg):
                d = (_lib.ARG_GLOBAL, int(a.access), as_code(a.data.dtype), a.data.cdim, -1, -1,
                     0, 0)
            elif isinstance(a, DatLegacyArg):
                mi = table.add(a.map_) if a.map_ is not None else -1
                d = (_lib.ARG_DAT, int(a.access), as_code(a.data.dtype), a.data.cdim, mi, -1, 0, 0)
            elif isinstance(a, MatLegacyArg):
                rm = table.add(a.maps[0])
                cm = table.add(a.maps[1])
                rdim, cdim = a.data.dims[0][0]
                d = (_lib.ARG_MAT, int(a.access), as_code(a.data.dtype), 1, rm, cm, rdim, cdim)
            elif isinstance(a, PassthroughArg):
                d = (_lib.ARG_PASSTHROUGH, int(Access.RW), as_code(a.dtype), 1, -1, -1, 0, 0)
            else:
                raise ValueError("Unhandled argument type %r" % type(a))
            stride = getattr(a.data, "_view_stride", 0) if isinstance(a, DatLegacyArg) else 0
            argdescs.append(d + (group, gcols, stride))
        return table, argdescs

    def _nc_reads(self):
        """True when no Dat read by a READ argument is written by another
        argument of this loop (READ gathers may then use the read-only path)."""
        read, written = set(), set()
        for a in self._components:
            if isinstance(a, DatLegacyArg):
                owner = a.data._parent if isinstance(a.data, DatView) else a.data
                (read if a.access is Access.READ else written).add(id(owner))
        return not (read & written)

    def _loop_desc(self, scatter, block_size, prefetch=None, cells=None):
        it = self.iterset
        if prefetch is None:
            prefetch = int(configuration["prefetch"])
        if cells is None:
            cells = int(configuration["cells_per_thread"])
        return dict(extruded=int(it._extruded),
                    constant_layers=int(bool(it._extruded and it.constant_layers)),
                    extruded_periodic=int(bool(it._extruded_periodic)),
                    indexed=int(isinstance(it, Subset) or scatter == _lib.SCATTER_PLAIN),
                    iteration_region=int(self.iteration_region),
                    pass_layer_arg=int(self.pass_layer_arg),
                    scatter=scatter, block_size=block_size,
                    debug_checks=int(bool(configuration["debug"])), batched=0,
                    prefetch=int(bool(prefetch) and not it._extruded),
                    nc_reads=int(self._nc_reads()),
                    cells_per_thread=max(1, int(cells)))

    def _needs_conflict_handling(self):
        return any(isinstance(a, (DatLegacyArg, MatLegacyArg)) and
                   (isinstance(a, MatLegacyArg) or a.map_ is not None) and
                   a.access in (Access.INC, Access.MIN, Access.MAX) for a in self._components)

    def _choose_strategy(self):
        """(scatter, block size, prefetch) from the configuration, or from
        the autotuner's measurements."""
        mode = configuration["scatter"]
        bs = int(configuration["block_size"])
        pf = int(configuration["prefetch"])
        grid = int(configuration["grid"])
        if mode == "auto" or configuration["autotune"]:
            from pyop2_gb300 import autotune
            return autotune.choose(self)
        if mode == "staged" and self._stageable():
            return _lib.SCATTER_STAGED, bs, pf, grid
        if not self._needs_conflict_handling():
            return _lib.SCATTER_ATOMIC, bs, pf, grid
        if mode == "warp":
            it = self.iterset
            if it._extruded and not it.constant_layers:
                return _lib.SCATTER_ATOMIC, bs, pf, grid
            return _lib.SCATTER_WARP, bs, pf, grid
        if mode == "colour" and self._colourable() and colour_plan(self) is not None:
            return _lib.SCATTER_PLAIN, bs, pf, grid
        if mode == "shared" and not self.iterset._extruded:
            return _lib.SCATTER_SHARED, bs, pf, grid
        return _lib.SCATTER_ATOMIC, bs, pf, grid

    def _stage_roots(self):
        """Plain maps (in first-seen order) whose staging plans a staged
        wrapper of this loop may read: those of Dat arguments (not parts of a
        mixed argument) through a plain or permuted map, READ or INC."""
        roots, seen = [], set()
        for a, group, _ in self._flat:
            if not isinstance(a, DatLegacyArg) or a.map_ is None or group:
                continue
            if a.access not in (Access.READ, Access.INC):
                continue
            m = a.map_
            if isinstance(m, PermutedMap):
                m = m.map_
            if isinstance(m, (ComposedMap, MixedMap)) or not isinstance(m, Map):
                continue
            if m._serial not in seen:
                seen.add(m._serial)
                roots.append(m)
        return roots

    def _stageable(self):
        """True when a staged wrapper applies: a non-extruded loop over a
        whole set with at least one Dat argument it can stage, whose staged
        values fit in shared memory."""
        it = self.iterset
        if it._extruded or isinstance(it, Subset) or not self._stage_roots():
            return False
        return stage_plan(self) is not None

    def _colourable(self):
        if self.iterset._extruded or isinstance(self.iterset, Subset):
            return False
        for a in self._components:
            if isinstance(a, DatLegacyArg) and a.map_ is not None and \
                    a.access in (Access.INC, Access.MIN, Access.MAX, Access.WRITE, Access.RW):
                if isinstance(a.map_, ComposedMap):
                    return False
            if isinstance(a, MatLegacyArg):
                if any(isinstance(m, ComposedMap) for m in a.maps):
                    return False
        return True

    def cache_key(self, scatter=_lib.SCATTER_ATOMIC, block_size=256):
        """Key of the compiled wrapper this loop uses (needs no device)."""
        table, argdescs = self._signature()
        return signature_key(self.local_kernel.source, self.local_kernel.name,
                             self._loop_desc(scatter, block_size), argdescs, table.key())

    def build(self, scatter=None, block_size=None, prefetch=None, grid=None, cells=None):
        """Compile the wrapper for this loop (idempotent per strategy).
        ``grid`` is the launch's CTA policy (``op2g_launch_desc.grid``),
        ``cells`` the iterations a thread runs per sweep step."""
        if scatter is None:
            choice = self._choose_strategy()
            scatter, block_size, prefetch, grid = choice[:4]
            if len(choice) > 4:
                cells = choice[4]
        if block_size is None:
            block_size = int(configuration["block_size"])
        self._grid = int(configuration["grid"]) if grid is None else int(grid)
        table, argdescs = self._signature()
        loop = self._loop_desc(scatter, block_size, prefetch, cells)
        k = compile_signature(self.local_kernel.source, self.local_kernel.name, loop, argdescs,
                              table.key())
        device.require()
        _lib.call("op2g_kernel_prepare", k.handle)   # module loaded outside any capture
        if scatter == _lib.SCATTER_STAGED and stage_plan(self) is None:
            raise ValueError("staged execution does not apply to this loop")
        self._built = (scatter, block_size, k, table, argdescs)
        self._launch_cache = None
        self._plan = None
        self._stage = None
        return k

    # ---- execution
    def _pointer_plan(self, table):
        """What the pointer slots come from, fixed for a built loop: per
        component its kind and object; the maps' device arrays (uploaded once,
        never moved) resolved now."""
        plan = []
        err = None
        for a in self._components:
            if isinstance(a, (GlobalLegacyArg, DatLegacyArg)):
                plan.append((0, a.data))
            elif isinstance(a, MatLegacyArg):
                plan.append((1, a.data))
                if err is None:
                    err = a.data._err
            elif isinstance(a, PassthroughArg):
                plan.append((2, int(a.data)))
        maps = [obj._device_values().data_ptr() if obj is not None else 0 for obj in table.objs]
        mats = [(a.data, Mat.ADD_VALUES if a.access is Access.INC else Mat.INSERT_VALUES)
                for a in self._components if isinstance(a, MatLegacyArg)]
        return plan, maps, err, mats

    def _pointers(self, table, k):
        """Device pointer slots (order documented in include/op2g.h) and the
        error-word pointer."""
        plan, maps, err, _ = self._plan
        ptrs = []
        for kind, obj in plan:
            if kind == 0:
                ptrs.append(obj._device_ptr())     # uploads host-side changes
            elif kind == 1:
                ptrs += [obj._values.data_ptr(), obj.sparsity.rowptr.data_ptr(),
                         obj.sparsity._colidx.data_ptr()]
            else:
                ptrs.append(obj)
        ptrs += maps
        assert len(ptrs) == k.nptrs
        return ptrs, err

    def _layers_per_entity(self):
        it = self.iterset
        if not (it._extruded and it.constant_layers):
            return 1
        L = int(it.layers_array[0, 1]) - int(it.layers_array[0, 0])   # layers
        ncell = L - 1
        r = self.iteration_region
        if r in (IterationRegion.BOTTOM, IterationRegion.TOP):
            return 1
        if r == IterationRegion.INTERIOR_FACETS and not it._extruded_periodic:
            return max(ncell - 1, 0)
        return ncell

    def __call__(self):
        self.compute()

    def launch_desc(self):
        """Synchronise the arguments to the device and return the launch
        descriptor of this loop (cached; pointer arrays kept alive on self).
        Also updates Mat assembly states as the reference does before a loop
        (pyop2/parloop.py:279-301)."""
        device.require()
        if self._built is None:
            self.build()
        scatter, bs, k, table, argdescs = self._built
        it = self.iterset
        if self._plan is None:
            self._plan = self._pointer_plan(table)
        for m, state in self._plan[3]:
            m.change_assembly_state(state)
        ptrs, err = self._pointers(table, k)
        dbg = configuration["debug"] and err is None
        cache = getattr(self, "_launch_cache", None)
        if cache is not None and cache[0] == ptrs and cache[1] == dbg:
            return cache[2]
        if dbg:
            self._dbg_err = torch.zeros(1, dtype=torch.int32, device=device.device())
            err = self._dbg_err
        else:
            self._dbg_err = None
        P = (ctypes.c_void_p * max(1, len(ptrs)))(*ptrs)
        toset = (ctypes.c_int64 * max(1, len(table.objs)))()
        for i in range(len(table.entries)):
            toset[i] = 2**62
        for a in self._components:
            if isinstance(a, DatLegacyArg) and a.map_ is not None:
                toset[table.add(a.map_)] = a.data.dataset.total_size
        D = _lib.LaunchDesc()
        D.layers = it._layers_device().data_ptr() if it._extruded else None
        D.err = err.data_ptr() if err is not None else None
        D.ptrs = P
        D.map_toset = toset
        D.layers_per_entity = self._layers_per_entity()
        D.grid = getattr(self, "_grid", 0)
        D.indices = it._indices_mirror.dev().data_ptr() if isinstance(it, Subset) else None
        D.start, D.end = 0, it.size
        if scatter == _lib.SCATTER_STAGED:
            if self._stage is None:
                self._stage = stage_plan(self)
            D.stage = ctypes.pointer(self._stage.desc(table))
        self._keep = (P, toset)
        self._launch_cache = (ptrs, dbg, D)
        return D

    def _written_lists(self):
        """What a launch leaves changed (pyop2/parloop.py:454-468), worked out
        once per set of arguments: Mats with their new assembly state, the
        Dats and Globals whose device copy becomes the newer one, and the
        Dats whose halos become stale."""
        mats, data, halos = [], [], []
        for a in self.args:
            if isinstance(a, MixedMatLegacyArg) and a.access is not Access.READ:
                mats.append((a.data, Mat.ADD_VALUES if a.access is Access.INC
                             else Mat.INSERT_VALUES))
        for a in self._components:
            if a.access is Access.READ or isinstance(a, PassthroughArg):
                continue
            if isinstance(a, MatLegacyArg):
                mats.append((a.data, Mat.ADD_VALUES if a.access is Access.INC
                             else Mat.INSERT_VALUES))
            else:
                data.append(a.data)
                if isinstance(a, DatLegacyArg):
                    halos.append(a.data)
        return mats, data, halos

    def mark_written(self):
        """State updates after a launch (pyop2/parloop.py:454-468)."""
        if self._written is None:
            self._written = self._written_lists()
        mats, data, halos = self._written
        for m, state in mats:
            m.assembly_state = state
            m.increment_dat_version()
        for d in data:
            d._m.dev_modified()
            d.increment_dat_version()
        for d in halos:
            d.halo_valid = False

    def compute(self):
        if configuration["profiling"]:
            from pyop2_gb300.profiling import timed_region
            # same region name as the reference's per-loop event
            # (pyop2/parloop.py:221-232)
            with timed_region("Parloop_%s_%s" % (self.iterset.name, self.local_kernel.name)):
                return self._compute()
        return self._compute()

    def _compute(self):
        self._enqueue(device.stream_handle())
        self.mark_written()
        if self._dbg_err is not None:
            e = int(self._dbg_err.item())
            if e & _lib.DEVERR_MAP_BOUNDS:
                self._dbg_err.zero_()
                raise MapValueError("par_loop %s: a map value is outside its target set"
                                    % self.local_kernel.name)

    # ---- graph capture (pyop2_gb300.graph.LoopGraph)
    def _prepare_capture(self):
        """Everything a launch does besides launching: build, upload, load the
        module, colour (none of it may happen inside a stream capture)."""
        self.launch_desc()          # also builds a staging plan
        _lib.call("op2g_kernel_prepare", self._built[2].handle)
        if self._built[0] == _lib.SCATTER_PLAIN:
            colour_plan(self)

    def _capture_key(self):
        return tuple(self._launch_cache[0])

    def _refresh(self):
        self.launch_desc()

    def _enqueue(self, st):
        """Launch this loop on stream `st` (no state updates)."""
        D = self.launch_desc()
        scatter, bs, k, table, argdescs = self._built
        if scatter == _lib.SCATTER_PLAIN:
            plan = colour_plan(self)
            start, end, idx = D.start, D.end, D.indices
            D.indices = plan.order.data_ptr()
            try:
                for c in range(plan.ncolours):
                    D.start, D.end = plan.ptr[c], plan.ptr[c + 1]
                    if D.end > D.start:
                        _lib.call("op2g_kernel_launch", k.handle, ctypes.byref(D), st)
            finally:
                D.start, D.end, D.indices = start, end, idx
        else:
            _lib.check(_launch(k.handle, ctypes.byref(D), st))

    def generated_source(self):
        """CUDA source of the wrapper this loop runs."""
        if self._built is None:
            self.build()
        return self._built[2].source()


def _launch(handle, desc, stream):
    """op2g_kernel_launch, bound once."""
    global _launch
    _launch = _lib.lib().op2g_kernel_launch
    return _launch(handle, desc, stream)


# ------------------------------------------------------------- colouring
class ColourPlan:
    """Greedy colouring of an iteration set w.r.t. the targets of its
    conflicting maps: ``order`` lists entities colour by colour,
    ``ptr[c]:ptr[c+1]`` is colour c's segment."""

    def __init__(self, order, ptr, ncolours, colour):
        self.order = order
        self.ptr = ptr
        self.ncolours = ncolours
        self.colour = colour

    def order_for_subset(self, subset_indices):
        raise NotImplementedError

    def validate(self, maps):
        """True if no two entities of one colour share a target through any
        of ``maps`` (the plan's correctness property; checked on the device)."""
        import torch
        for c in range(self.ncolours):
            seg = self.order[self.ptr[c]:self.ptr[c + 1]].long()
            if seg.numel() == 0:
                continue
            if not bool((self.colour[seg] == c).all()):
                return False
            for m in maps:
                vals = m._device_values()[:m.values_with_halo.nbytes].view(torch.int32)
                t = vals.view(-1, m.arity)[seg]
                # a cell may name one target twice: count each target once per cell
                t, _ = torch.sort(t, dim=1)
                t[:, 1:][t[:, 1:] == t[:, :-1]] = -1
                t = t.reshape(-1)
                t = t[t >= 0]
                if torch.unique(t).numel() != t.numel():
                    return False
        return True


def colour_plan(loop, max_colours=256):
    """Colouring of ``loop.iterset`` (cached on the set per tuple of written
    maps)."""
    it = loop.iterset
    if isinstance(it, Subset):
        raise NotImplementedError("coloured execution of subsets")
    maps = []
    for a in loop._components:
        if a.access is Access.READ:
            continue
        if isinstance(a, DatLegacyArg) and a.map_ is not None:
            maps.append(a.map_)
        elif isinstance(a, MatLegacyArg):
            maps.extend(a.maps)
    base = []
    seen = set()
    for m in maps:
        b = m.map_ if isinstance(m, PermutedMap) else m
        if b._serial not in seen:
            seen.add(b._serial)
            base.append(b)
    # keyed by the maps' serial numbers (never reused, unlike id()); the
    # values of a map are fixed once on the device, so the plan stays valid
    key = ("colour", tuple(b._serial for b in base))
    if key in it._cache:
        return it._cache[key]
    n = it.size
    dev = device.device()
    arrs = (ctypes.c_void_p * len(base))(*[b._device_values().data_ptr() for b in base])
    ar = (ctypes.c_int32 * len(base))(*[b.arity for b in base])
    tsz = (ctypes.c_int64 * len(base))(*[b.toset.total_size for b in base])
    ws = ctypes.c_size_t()
    _lib.call("op2g_colour_workspace", n, len(base), tsz, ctypes.byref(ws))
    work = device.empty_bytes(ws.value)
    colour = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    order = torch.empty(max(n, 1), dtype=torch.int32, device=dev)
    cptr = torch.empty(max_colours + 1, dtype=torch.int64, device=dev)
    nc = ctypes.c_int32()
    st = _lib.lib().op2g_colour(n, len(base), arrs, ar, tsz, max_colours, work.data_ptr(),
                                ws.value, colour.data_ptr(), order.data_ptr(), cptr.data_ptr(),
                                ctypes.byref(nc), device.stream_handle())
    if st == _lib.ERR_CAPACITY:
        # more than max_colours colours: the loop falls back to atomics
        it._cache[key] = None
        return None
    _lib.check(st)
    ptr = cptr[:nc.value + 1].cpu().numpy().tolist()
    plan = ColourPlan(order, ptr, nc.value, colour)
    it._cache[key] = plan
    return plan


# ---------------------------------------------------------- staging plans
class MapStagePlan:
    """The staging plan of one map over its iteration set's ``size`` entities:
    partitions of ``block`` iterations; per partition a segment (at
    ``ind_off[p]``, 16-byte aligned) of its ``ind_num[p]`` sorted distinct
    targets (``ind_map``) with the first slot of each (``run_off``), and per
    map entry its slot (``loc_map``, uint16: its rank in the partition's
    entries sorted by target; 0xFFFF for a negative entry) -- the local
    renumbering of the historical OP2 execution plan
    (doc/sphinx/source/plan.rst:21-39), built on the device."""

    def __init__(self, m, block):
        n, ar = m.iterset.size, m.arity
        dev = device.device()
        nb = (n + block - 1) // block
        st = device.stream_handle()
        vals = m._device_values()
        ws = ctypes.c_size_t()
        _lib.call("op2g_stage_plan_workspace", n, ar, block, ctypes.byref(ws))
        work = device.empty_bytes(ws.value)
        self.ind_off = torch.empty(nb + 1, dtype=torch.int64, device=dev)
        self.ind_num = torch.empty(max(nb, 1), dtype=torch.int32, device=dev)
        total = ctypes.c_int64()
        mx = ctypes.c_int32()
        _lib.call("op2g_stage_plan_count", n, ar, vals.data_ptr(), block, work.data_ptr(),
                  ws.value, self.ind_off.data_ptr(), self.ind_num.data_ptr(), ctypes.byref(total),
                  ctypes.byref(mx), st)
        self.ind_map = torch.empty(max(total.value, 8), dtype=torch.int32, device=dev)
        self.run_off = torch.empty(max(total.value, 8), dtype=torch.int16, device=dev)
        # 16-byte bulk copies of a partition's slots may read up to 7 entries
        # past the last one
        self.loc_map = torch.empty(n * ar + 8, dtype=torch.int16, device=dev)
        _lib.call("op2g_stage_plan_fill", n, ar, vals.data_ptr(), block,
                  self.ind_off.data_ptr(), self.ind_map.data_ptr(), self.run_off.data_ptr(),
                  self.loc_map.data_ptr(), st)
        self.n = n
        self.block = block
        self.max_unique = mx.value
        self.total = total.value
        self.nblocks = nb


class StagePlan:
    """The staging plans of a loop's maps, all with one partition size."""

    def __init__(self, plans, block, n):
        self.plans = plans          # map serial -> MapStagePlan
        self.block = block
        self.n = n                  # iterations covered
        self._descs = {}

    def desc(self, table):
        """op2g_stage_desc for the loop's map table (entries in table order)."""
        key = tuple(id(o) for o in table.objs)
        d = self._descs.get(key)
        if d is None:
            d = _lib.StageDesc()
            d.block = self.block
            d.n = self.n
            for i, obj in enumerate(table.objs):
                mp = self.plans.get(obj._serial) if obj is not None else None
                if mp is None:
                    continue
                d.ind_map[i] = mp.ind_map.data_ptr()
                d.ind_off[i] = mp.ind_off.data_ptr()
                d.ind_num[i] = mp.ind_num.data_ptr()
                d.run_off[i] = mp.run_off.data_ptr()
                d.loc_map[i] = mp.loc_map.data_ptr()
                d.max_unique[i] = mp.max_unique
            self._descs[key] = d
        return d


_STAGE_SMEM_LIMIT = 200 * 1024


def stage_plan(loop):
    """Staging plan of a loop's stageable maps (cached on each map per
    partition size), or None when its staged values would not fit in shared
    memory.  The partition size is configuration["stage_cells"], capped at
    4096 map entries per partition and rounded down to a multiple of 32."""
    roots = loop._stage_roots()
    if not roots:
        return None
    arity = max(m.arity for m in roots)
    block = min(int(configuration["stage_cells"]), 4096 // arity)
    block = max(32, block - block % 32)
    if 4096 // arity < 32:
        return None
    plans = {}
    for m in roots:
        key = ("stage", block, m.iterset.size)
        mp = m._cache.get(key)
        if mp is None:
            mp = MapStagePlan(m, block)
            m._cache[key] = mp
        plans[m._serial] = mp
    # shared memory of the staged wrapper (an upper bound of what it takes):
    # per staged map three plan buffers (target list, run offsets, slots) and
    # the slot -> target table; per READ argument two buffers of values per
    # target, per INC argument one value per slot; per direct READ argument
    # two buffers of the partition's values
    def r16(x):
        return (x + 15) // 16 * 16
    smem = 0
    for m in roots:
        mu = plans[m._serial].max_unique
        seg = (mu + 1 + 7) // 8 * 8
        smem += 3 * (r16(seg * 4) + r16(seg * 2) + r16(block * m.arity * 2)) + \
            r16(block * m.arity * 2)
    for a, group, _ in loop._flat:
        if not isinstance(a, DatLegacyArg) or group:
            continue
        size = a.data.cdim * a.data.dtype.itemsize
        if a.map_ is None:
            if a.access is Access.READ:
                smem += 2 * r16(block * size)
            continue
        m = a.map_.map_ if isinstance(a.map_, PermutedMap) else a.map_
        if m._serial in plans and a.access in (Access.READ, Access.INC):
            smem += 2 * r16(plans[m._serial].max_unique * size) if a.access is Access.READ \
                else r16(block * m.arity * size)
    if smem > _STAGE_SMEM_LIMIT:
        return None
    return StagePlan(plans, block, loop.iterset.size)


# ------------------------------------------------------------ entry points
def LegacyParloop(local_knl, iterset, *args, **kwargs):
    """Build a Parloop from legacy arguments (pyop2/parloop.py:707-741)."""
    if not all(isinstance(a, LegacyArg) for a in args):
        raise ValueError("LegacyParloop only expects LegacyArg arguments")
    if not isinstance(iterset, Set):
        raise SetTypeError("Iteration set is of the wrong type")
    local_knl.accesses = tuple(a.access for a in args)
    if isinstance(local_knl, CStringLocalKernel):
        local_knl.dtypes = tuple(a.dtype for a in args)
    return Parloop(local_knl, iterset, args, **kwargs)


def global_kernel_of(local_knl, iterset, args, iteration_region=None, pass_layer_arg=False):
    """The GlobalKernel describing a legacy loop (pyop2/parloop.py:719-737)."""
    from pyop2_gb300.global_kernel import GlobalKernel
    extruded = iterset._extruded
    return GlobalKernel(local_knl, tuple(a.global_kernel_arg for a in args),
                        extruded=extruded,
                        extruded_periodic=iterset._extruded_periodic,
                        constant_layers=bool(extruded and iterset.constant_layers),
                        subset=isinstance(iterset, Subset),
                        iteration_region=iteration_region, pass_layer_arg=pass_layer_arg)


def ParLoop(*args, **kwargs):
    return LegacyParloop(*args, **kwargs)


# Recently run loops, so that a par_loop call repeating an earlier one (same
# kernel, iteration set, data objects, maps, access modes and options) skips
# validation and signature building and reuses the launch descriptor (the
# host cost of a call drops from ~45 to ~12 us, which is what a loop over a
# few thousand cells costs on the device).  The entries hold their objects,
# so the ids in a key cannot be reused while it lives; the cost is that their
# data stay alive.  That is bounded: at most 16 entries, whose Dat / Mat /
# Global data together take at most configuration["recent_loops_bytes"]
# (least recently used entries go first; a loop whose own data exceed the
# bound is not kept).  Loops made internally for temporaries (Dat
# arithmetic) go through run_once and are not kept.
_RECENT = collections.OrderedDict()     # key -> (loop, kernel, iterset, bytes)
_RECENT_SIZE = 16
_RECENT_BYTES = [0]
_CONFIG_KEYS = ("scatter", "block_size", "prefetch", "grid", "debug", "autotune", "type_check")


def _data_bytes(args):
    """Bytes of the distinct Dat / Mat / Global objects a loop references."""
    seen, total = set(), 0
    for a in args:
        objs = a.data if isinstance(a, (MixedDatLegacyArg,)) else (
            getattr(a, "data", None),)
        for o in objs:
            if o is None or isinstance(o, int) or id(o) in seen:
                continue
            seen.add(id(o))
            total += int(getattr(o, "nbytes", 0) or 0)
    return total


def _recent_drop_oldest():
    _, hit = _RECENT.popitem(last=False)
    _RECENT_BYTES[0] -= hit[3]


def recent_loops_clear():
    """Forget every remembered loop (their data are no longer kept alive)."""
    _RECENT.clear()
    _RECENT_BYTES[0] = 0


def _arg_key(a):
    if isinstance(a, DatLegacyArg):
        return (0, id(a.data), id(a.map_), a.access)
    if isinstance(a, GlobalLegacyArg):
        return (1, id(a.data), a.access)
    if isinstance(a, MatLegacyArg):
        return (2, id(a.data), id(a.maps[0]), id(a.maps[1]), a.access, a.needs_unrolling)
    if isinstance(a, MixedDatLegacyArg):
        return (3, id(a.data), id(a.map_), a.access)
    if isinstance(a, MixedMatLegacyArg):
        return (4, id(a.data), id(a.maps[0]), id(a.maps[1]), a.access)
    if isinstance(a, PassthroughArg):
        return (5, a.data, repr(a.dtype))
    return None


def parloop(knl, *args, **kwargs):
    """Construct and execute a par_loop (pyop2/parloop.py:748-760)."""
    if not isinstance(knl, LocalKernel):
        raise KernelTypeError
    key = None
    if args:
        akeys = tuple(_arg_key(a) for a in args[1:])
        if None not in akeys:
            try:
                key = (id(knl), id(knl.code), id(args[0]), akeys, tuple(sorted(kwargs.items())),
                       tuple(configuration[k] for k in _CONFIG_KEYS))
                hash(key)
            except TypeError:      # an unhashable keyword value: no reuse
                key = None
    pl = None
    if key is not None:
        hit = _RECENT.get(key)
        if hit is not None and hit[1] is knl and hit[2] is args[0]:
            pl = hit[0]
            _RECENT.move_to_end(key)
            for a in pl._components:      # halo freezing can change between calls
                if isinstance(a, DatLegacyArg) and a.data._halo_frozen and \
                        a.data._frozen_access_mode != a.access:
                    raise RuntimeError("Dats with frozen halos must always be accessed with "
                                       "the same access mode")
    if pl is None:
        pl = LegacyParloop(knl, *args, **kwargs)
        if key is not None:
            nb = _data_bytes(args[1:])
            limit = int(configuration["recent_loops_bytes"])
            if nb <= limit:
                old = _RECENT.pop(key, None)
                if old is not None:
                    _RECENT_BYTES[0] -= old[3]
                while _RECENT and (len(_RECENT) >= _RECENT_SIZE or
                                   _RECENT_BYTES[0] + nb > limit):
                    _recent_drop_oldest()
                _RECENT[key] = (pl, knl, args[0], nb)
                _RECENT_BYTES[0] += nb
    pl()


def run_once(knl, *args, **kwargs):
    """Run a loop without keeping it for reuse."""
    if not isinstance(knl, LocalKernel):
        raise KernelTypeError
    LegacyParloop(knl, *args, **kwargs)()


def par_loop(*args, **kwargs):
    parloop(*args, **kwargs)
