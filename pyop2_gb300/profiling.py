"""Named timed regions (pyop2/profiling.py:39-61).

The reference wraps its work in PETSc log events (``Parloop_<set>_<kernel>``,
``CreateSparsity``, ``MatZeroInitial`` ...).  Here a region is an NVTX range
(visible in Nsight tools) and, when ``configuration['profiling']`` is on, a
pair of CUDA events on the current stream whose elapsed device time is
accumulated per region name.  ``summary()`` synchronises and returns
{name: (calls, total device ms)}.
"""
import contextlib

from pyop2_gb300.configuration import configuration

_pending = []     # (name, start event, end event)
_totals = {}      # name -> [calls, ms]


def _nvtx():
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.nvtx
    except Exception:
        pass
    return None


@contextlib.contextmanager
def timed_region(name):
    """NVTX range + (optionally) device timing of the enclosed launches."""
    if not configuration["profiling"]:
        yield
        return
    import torch
    nv = _nvtx()
    if nv is not None:
        nv.range_push(name)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    try:
        yield
    finally:
        e1.record()
        _pending.append((name, e0, e1))
        if nv is not None:
            nv.range_pop()


def timed_function(name=None):
    """Decorator form of timed_region."""
    def deco(f):
        n = name or f.__name__

        def wrapper(*a, **k):
            with timed_region(n):
                return f(*a, **k)
        wrapper.__name__ = f.__name__
        wrapper.__doc__ = f.__doc__
        return wrapper
    return deco


def _drain():
    while _pending:
        name, e0, e1 = _pending.pop(0)
        e1.synchronize()
        t = _totals.setdefault(name, [0, 0.0])
        t[0] += 1
        t[1] += e0.elapsed_time(e1)


def summary():
    """{region name: (calls, device milliseconds)} accumulated so far."""
    _drain()
    return {k: (v[0], v[1]) for k, v in _totals.items()}


def reset():
    _drain()
    _totals.clear()
