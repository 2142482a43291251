"""CUDA graphs of par_loops (``op2g_graph_begin`` / ``op2g_graph_end``).

``LoopGraph(loops)`` records the launches of ``loops`` -- ParLoops (any INC
strategy; a coloured loop records one launch per colour) and
BatchedParLoops -- once, in order, into an instantiated CUDA graph;
``replay()`` runs them as one unit with a single launch call.  This is the
GPU-native form of a solver step that repeats the same loops: the per-loop
host work (validation, descriptors, launch calls) is paid once.  There is no
counterpart in the reference (each par_loop is a separate call).

A replay uses the device arrays the loops referenced when they were
recorded.  Host-side changes to the loops' Dats are uploaded before each
replay (into the same arrays); if an argument's device array itself changed,
the graph is recorded again.  Debug-mode map bounds checks are not read
back after a replay.
"""
import ctypes

from pyop2_gb300 import _lib, device


class LoopGraph:
    def __init__(self, loops):
        if not loops:
            raise ValueError("LoopGraph needs at least one loop")
        self.loops = list(loops)
        # a loop recorded several times is refreshed and marked once per replay
        self._distinct = list({id(lp): lp for lp in self.loops}.values())
        self.handle = None
        self._record()

    def _record(self):
        self._destroy()
        for lp in self._distinct:
            lp._prepare_capture()
        self._keys = [lp._capture_key() for lp in self._distinct]
        s = ctypes.c_void_p()
        _lib.call("op2g_graph_begin", ctypes.byref(s))
        failure = None
        try:
            for lp in self.loops:
                lp._enqueue(s)
        except BaseException as e:       # the capture is ended below either way
            failure = e
        h = ctypes.c_void_p()
        try:
            _lib.call("op2g_graph_end", s, ctypes.byref(h))
        except BaseException as e:
            if failure is None:
                failure = e
        if failure is not None:
            raise failure
        self.handle = h

    def launch(self, stream=None):
        """Run the recorded launches on `stream` (default: the current
        stream) without any host-side bookkeeping."""
        _lib.call("op2g_graph_launch", self.handle,
                  device.stream_handle() if stream is None else stream)

    def replay(self):
        """Upload host-side changes, run the graph, mark the written
        arguments (re-recording first if an argument moved)."""
        for lp in self._distinct:
            lp._refresh()
        if [lp._capture_key() for lp in self._distinct] != self._keys:
            self._record()
        self.launch()
        for lp in self._distinct:
            lp.mark_written()

    def _destroy(self):
        if self.handle:
            _lib.lib().op2g_graph_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self._destroy()
        except Exception:
            pass
