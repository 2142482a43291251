"""Runtime configuration, mirroring pyop2/configuration.py:43-172.

Kept keys use the reference's ``PYOP2_*`` environment variables; keys that
only exist here use ``OP2G_*``.
"""
import os
from tempfile import gettempdir

from pyop2_gb300.exceptions import ConfigurationError


def _bool(v):
    if isinstance(v, str):
        return v.strip().lower() not in ("", "0", "false", "no", "off")
    return bool(v)


class Configuration(dict):
    # name: (environment variable, type, default)
    DEFAULTS = {
        "debug": ("PYOP2_DEBUG", bool, False),
        "type_check": ("PYOP2_TYPE_CHECK", bool, True),
        "log_level": ("PYOP2_LOG_LEVEL", (str, int), "WARNING"),
        "cache_dir": ("PYOP2_CACHE_DIR", str,
                      os.path.join(gettempdir(), "pyop2_gb300-cache-uid%s" % os.getuid())),
        "block_sparsity": ("PYOP2_BLOCK_SPARSITY", bool, True),
        "matnest": ("PYOP2_MATNEST", bool, True),
        "compute_kernel_flops": ("PYOP2_COMPUTE_KERNEL_FLOPS", bool, False),
        "print_cache_info": ("PYOP2_CACHE_INFO", bool, False),
        # INC conflict resolution: "atomic", "warp", "colour", "shared" (per-CTA
        # shared-memory sums, one atomic per distinct target), "staged" (a
        # staging plan: READ and INC data of each mini-partition in shared
        # memory at its distinct targets) or "auto" (autotuner)
        "scatter": ("OP2G_SCATTER", str, "atomic"),
        # iterations each thread runs per sweep step, their gathers and
        # arithmetic interleaved (1 or 2)
        "cells_per_thread": ("OP2G_CELLS_PER_THREAD", int, 1),
        # iterations per mini-partition of a staging plan (at most 4096 / arity)
        "stage_cells": ("OP2G_STAGE_CELLS", int, 512),
        # threads per CTA of generated wrappers
        "block_size": ("OP2G_BLOCK_SIZE", int, 256),
        # let the autotuner pick scatter strategy, block size and prefetch per kernel
        "autotune": ("OP2G_AUTOTUNE", bool, False),
        # generated wrappers load the next iteration's map rows ahead (0 or 1)
        "prefetch": ("OP2G_PREFETCH", int, 0),
        # CTAs per launch: 0 = one per block of iterations up to 4 resident
        # waves (threads stride over the rest), -1 = one per block, no cap
        "grid": ("OP2G_GRID", int, 0),
        # CUDA device used by this process
        "device": ("OP2G_DEVICE", int, 0),
        # NVTX ranges + CUDA-event timing of named regions (profiling.summary())
        "profiling": ("OP2G_PROFILING", bool, False),
        # check a Map's values against its target set when they are uploaded
        # (an index outside it would fault the GPU; with "debug" the launch
        # checks every access instead)
        "check_maps": ("OP2G_CHECK_MAPS", bool, True),
        # bytes of Dat / Mat / Global data that op2.par_loop's table of
        # recently run loops may keep alive; a loop whose own data exceed it is
        # not kept (deleting its data then frees the device memory)
        "recent_loops_bytes": ("OP2G_RECENT_LOOPS_BYTES", int, 1 << 30),
    }

    def __init__(self):
        super().__init__()
        self._set = set()
        self.reset()

    def reset(self):
        for k, (env, typ, default) in self.DEFAULTS.items():
            v = os.environ.get(env)
            if v is None:
                self[k] = default
            else:
                self[k] = self._convert(k, v)

    def _convert(self, key, value):
        typ = self.DEFAULTS[key][1]
        if typ is bool:
            return _bool(value)
        if typ is int:
            return int(value)
        if isinstance(typ, tuple):
            return value
        return typ(value)

    def reconfigure(self, **kwargs):
        for k, v in kwargs.items():
            self[k] = v

    def __setitem__(self, key, value):
        """Known keys are type-checked (pyop2/configuration.py:155-168: a value
        of the wrong type raises ConfigurationError); other keys are stored."""
        if key in self.DEFAULTS:
            typ = self.DEFAULTS[key][1]
            ok = isinstance(value, typ) if isinstance(typ, tuple) else (
                isinstance(value, bool) if typ is bool else
                isinstance(value, int) and not isinstance(value, bool) if typ is int else
                isinstance(value, typ))
            if not ok:
                raise ConfigurationError("Values for configuration key %s must be of type %r, "
                                         "not %r" % (key, typ, type(value)))
        if key == "scatter" and value not in ("atomic", "warp", "colour", "shared", "staged",
                                              "auto"):
            raise ConfigurationError("scatter must be atomic, warp, colour, shared, staged or "
                                     "auto")
        self._set.add(key)
        super().__setitem__(key, value)


configuration = Configuration()
