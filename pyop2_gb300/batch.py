"""Many par_loops in one persistent launch, optionally replayed from a CUDA
graph.

All loops must share one signature (same kernel, argument kinds, access
modes, dims and map shapes) -- e.g. the same operator on many meshes of
uneven size.  Each loop contributes a parameter record (its device
pointers); its iteration range is cut into chunks, and the CTAs of one
launch of the wrapper's batched entry point take (loop, chunk) work items
round robin (``op2g_kernel_launch_batched``).  This removes the per-launch
cost and the tail of each small launch that dominate when most meshes are
small.  There is no counterpart in the reference (it runs one loop per
call).
"""
import ctypes

import numpy as np
import torch

from pyop2_gb300 import _lib, device
from pyop2_gb300.configuration import configuration


class BatchedParLoop:
    """``BatchedParLoop(parloops, chunk=2048, block_size=None, scatter=None)``

    ``compute()`` runs every loop once (one kernel launch); ``capture()``
    records that launch into a CUDA graph and ``replay()`` runs the graph.
    """

    def __init__(self, loops, chunk=2048, block_size=None, scatter=None):
        if not loops:
            raise ValueError("BatchedParLoop needs at least one loop")
        self.loops = list(loops)
        self.chunk = int(chunk)
        self.block_size = int(block_size or configuration["block_size"])
        self.scatter = _lib.SCATTER_ATOMIC if scatter is None else scatter
        if self.scatter == _lib.SCATTER_PLAIN:
            raise ValueError("coloured execution cannot be batched")
        self._graph = None
        self._build()

    def _build(self):
        device.require()
        first = self.loops[0]
        sig0 = first._signature()
        key0 = (first.local_kernel.source, first.local_kernel.name, sig0[0].key(), tuple(sig0[1]))
        for lp in self.loops[1:]:
            sg = lp._signature()
            key = (lp.local_kernel.source, lp.local_kernel.name, sg[0].key(), tuple(sg[1]))
            if key != key0 or lp.iteration_region != first.iteration_region or \
                    lp.pass_layer_arg != first.pass_layer_arg or \
                    type(lp.iterset) is not type(first.iterset):
                raise ValueError("all loops of a batch need the same signature")
        k = None
        for lp in self.loops:
            k = lp.build(self.scatter, self.block_size)
        self.kernel = k
        L = _lib.lib()
        rec = L.op2g_kernel_param_bytes(k.handle)
        self.record_bytes = rec
        host = np.zeros(len(self.loops) * rec, dtype=np.uint8)
        work = []
        for i, lp in enumerate(self.loops):
            D = lp.launch_desc()
            _lib.check(L.op2g_kernel_pack_params(k.handle, ctypes.byref(D),
                                                 host[i * rec:].ctypes.data))
            n = lp.iterset.size
            for s in range(0, n, self.chunk):
                work.append((i, s, min(n, s + self.chunk)))
        # large chunks first is unnecessary (chunks are uniform); interleave
        # loops so that concurrent CTAs touch different meshes
        work.sort(key=lambda w: (w[1], w[0]))
        dev = device.device()
        self.params = torch.from_numpy(host).to(dev)
        self.work = torch.tensor(np.asarray(work, dtype=np.int64).reshape(-1), device=dev)
        self.nwork = len(work)

    def compute(self):
        """Run every loop once in one launch."""
        self._enqueue(device.stream_handle())
        self.mark_written()

    def capture(self):
        """Record the launch into a CUDA graph (pyop2_gb300.graph.LoopGraph;
        replay() runs it)."""
        from pyop2_gb300.graph import LoopGraph
        self._graph = LoopGraph([self])
        return self._graph

    def replay(self):
        if self._graph is None:
            self.capture()
        self._graph.replay()

    # ---- graph capture
    def _prepare_capture(self):
        self._refresh()
        _lib.call("op2g_kernel_prepare", self.kernel.handle)

    def _capture_key(self):
        return (self.params.data_ptr(), self.work.data_ptr(), self.nwork)

    def _refresh(self):
        for lp in self.loops:
            lp.launch_desc()     # uploads any host-side changes

    def _enqueue(self, st):
        self._refresh()
        _lib.call("op2g_kernel_launch_batched", self.kernel.handle, self.params.data_ptr(),
                  self.work.data_ptr(), self.nwork, 0, st)

    def mark_written(self):
        for lp in self.loops:
            lp.mark_written()


def autotune_batch(loops, chunks=(512, 2048, 8192), block_sizes=(128, 256), reps=3,
                   scatters=None):
    """Pick the (chunk, block size, INC strategy) of a batch by timing graph
    replays on the loops' own data; the written arguments are restored after
    each trial.  Strategies: hardware atomics, warp aggregation and
    shared-memory staging (colouring cannot run in one launch)."""
    if scatters is None:
        scatters = (_lib.SCATTER_ATOMIC,)
        if loops[0]._needs_conflict_handling():
            scatters = (_lib.SCATTER_ATOMIC, _lib.SCATTER_WARP)
            if not loops[0].iterset._extruded:
                scatters += (_lib.SCATTER_SHARED,)
    from pyop2_gb300.autotune import _restore, _snapshot, _written
    objs = []
    seen = set()
    for lp in loops:
        for o in _written(lp):
            if id(o) not in seen:
                seen.add(id(o))
                objs.append(o)
    snaps = _snapshot(objs)
    best = None
    trials = [(bs, ch, sc) for sc in scatters for bs in block_sizes for ch in chunks]
    for bs, ch, sc in trials:
        b = BatchedParLoop(loops, chunk=ch, block_size=bs, scatter=sc)
        b.capture()
        b.replay()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            b._graph.launch()
        e1.record()
        e1.synchronize()
        t = e0.elapsed_time(e1) / reps
        _restore(snaps)
        if best is None or t < best[0]:
            best = (t, ch, bs, b, sc)
    for o, t, s in snaps:
        if hasattr(o, "_m"):
            o._m.state = "device"
    names = {_lib.SCATTER_ATOMIC: "atomic", _lib.SCATTER_WARP: "warp",
             _lib.SCATTER_SHARED: "shared"}
    return best[3], {"chunk": best[1], "block_size": best[2], "scatter": names[best[4]],
                     "ms": best[0]}
