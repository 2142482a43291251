"""Autotuner: picks the INC conflict strategy and CTA size per loop signature
by timing the candidates on the loop's own data (with the written arguments
saved and restored around each trial).  Results are cached per
(kernel, signature, problem size)."""
import torch

from pyop2_gb300 import _lib, device
from pyop2_gb300.types.access import Access

_CHOICES = {}


def candidates(loop):
    """(scatter, block size, prefetch, grid[, cells per thread]) tuples worth timing for this
    loop: every INC strategy that applies (atomics, warp aggregation,
    shared-memory hash tables, colouring, a staging plan), three CTA sizes,
    for non-extruded
    loops the map-row prefetch on and off (the staging depth), and the two
    grid policies (up to 4 resident waves, or one CTA per block of cells)."""
    it = loop.iterset
    pfs = (0, 1) if not it._extruded else (0,)
    out = []
    staged = loop._stageable()
    for bs in (128, 256, 512):
        if staged:
            # staged partitions take their partition in turn; prefetch and the
            # grid policy do not apply
            out.append((_lib.SCATTER_STAGED, bs, 0, 0))
        for grid in (0, -1):
            # two cells per thread, interleaved (no prefetch)
            out.append((_lib.SCATTER_ATOMIC, bs, 0, grid, 2))
        for pf in pfs:
            for grid in (0, -1):
                out.append((_lib.SCATTER_ATOMIC, bs, pf, grid))
                if loop._needs_conflict_handling():
                    if not (it._extruded and not it.constant_layers):
                        out.append((_lib.SCATTER_WARP, bs, pf, grid))
                    if not it._extruded:
                        out.append((_lib.SCATTER_SHARED, bs, pf, grid))
                    if loop._colourable():
                        from pyop2_gb300.parloop import colour_plan
                        if colour_plan(loop) is not None:
                            out.append((_lib.SCATTER_PLAIN, bs, pf, grid))
    return out


def _written(loop):
    out = []
    for a in loop._components:
        if a.access is Access.READ or not hasattr(a.data, "_m") and not hasattr(a.data, "_values"):
            continue
        out.append(a.data)
    return out


def _snapshot(objs):
    snaps = []
    for o in objs:
        t = o._m.dev() if hasattr(o, "_m") else o._values
        snaps.append((o, t, t.clone()))
    return snaps


def _restore(snaps):
    for o, t, s in snaps:
        t.copy_(s)


def choose(loop, reps=3):
    key = (loop.local_kernel.cache_key[0], loop._signature()[1].__repr__(), loop.iterset.size,
           type(loop.iterset).__name__)
    if key in _CHOICES:
        return _CHOICES[key]
    device.require()
    cands = candidates(loop)
    if len(cands) == 1:
        _CHOICES[key] = cands[0]
        return cands[0]
    snaps = _snapshot(_written(loop))
    best = None
    for cand in cands:
        loop.build(*cand)
        loop.compute()   # warm-up (and compilation, colouring plan)
        _restore(snaps)
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        times = []
        for _ in range(reps):
            ev0.record()
            loop.compute()
            ev1.record()
            ev1.synchronize()
            times.append(ev0.elapsed_time(ev1))
            _restore(snaps)
        t = min(times)
        if best is None or t < best[0]:
            best = (t, tuple(cand))
    loop._built = None
    for o, t, s in snaps:
        if hasattr(o, "_m"):
            o._m.state = "device"
    _CHOICES[key] = best[1]
    return best[1]
