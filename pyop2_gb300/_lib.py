"""ctypes binding of libop2g.so (declarations in include/op2g.h).

The structures below mirror the C ABI field by field.  Loading the library
needs no GPU; launching anything does.  There is no fallback: if the library
is missing, every entry point raises.
"""
import ctypes
import os

from pyop2_gb300.exceptions import CompilationError

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libop2g.so")

OK = 0
ERR_INVALID, ERR_COMPILE, ERR_CUDA, ERR_BOUNDS, ERR_NEW_NONZERO, ERR_CAPACITY, \
    ERR_UNSUPPORTED, ERR_TIMEOUT = range(1, 9)
DEVERR_MAP_BOUNDS, DEVERR_NEW_NONZERO, DEVERR_CAPACITY = 1, 2, 4

F64, F32, I32, U32, I64, U64, I16, U16, I8, U8 = range(10)
ABI_VERSION = 4
ARG_DAT, ARG_GLOBAL, ARG_MAT, ARG_PASSTHROUGH = range(4)
MAP_PLAIN, MAP_PERMUTED, MAP_COMPOSED = range(3)
SCATTER_ATOMIC, SCATTER_WARP, SCATTER_PLAIN, SCATTER_SHARED, SCATTER_STAGED = range(5)
MAX_ARGS = 32
MAX_MAPS = 32
MAX_COMPOSED = 8

_i32 = ctypes.c_int32
_i64 = ctypes.c_int64
_p = ctypes.c_void_p
_pi32 = ctypes.POINTER(ctypes.c_int32)


class MapDesc(ctypes.Structure):
    _fields_ = [("kind", _i32), ("arity", _i32), ("base", _i32), ("ncomposed", _i32),
                ("composed", _i32 * MAX_COMPOSED), ("offset", _pi32),
                ("offset_quotient", _pi32), ("permutation", _pi32)]


class ArgDesc(ctypes.Structure):
    _fields_ = [("kind", _i32), ("access", _i32), ("dtype", _i32), ("dim", _i32),
                ("map", _i32), ("cmap", _i32), ("rdim", _i32), ("cdim", _i32),
                ("group", _i32), ("group_cols", _i32), ("stride", _i32)]


class LoopDesc(ctypes.Structure):
    _fields_ = [("extruded", _i32), ("constant_layers", _i32), ("extruded_periodic", _i32),
                ("indexed", _i32), ("iteration_region", _i32), ("pass_layer_arg", _i32),
                ("scatter", _i32), ("block_size", _i32), ("debug_checks", _i32),
                ("batched", _i32), ("prefetch", _i32), ("nc_reads", _i32),
                ("cells_per_thread", _i32)]


class StageDesc(ctypes.Structure):
    _fields_ = [("block", _i64), ("n", _i64), ("ind_map", _p * MAX_MAPS), ("ind_off", _p * MAX_MAPS),
                ("ind_num", _p * MAX_MAPS), ("run_off", _p * MAX_MAPS),
                ("loc_map", _p * MAX_MAPS), ("max_unique", _i32 * MAX_MAPS)]


class LaunchDesc(ctypes.Structure):
    _fields_ = [("start", _i64), ("end", _i64), ("layers", _p), ("indices", _p), ("err", _p),
                ("ptrs", ctypes.POINTER(_p)), ("map_toset", ctypes.POINTER(_i64)),
                ("layers_per_entity", _i64), ("grid", _i32), ("stage", ctypes.POINTER(StageDesc))]


class SparsityPair(ctypes.Structure):
    _fields_ = [("rmap", _p), ("cmap", _p), ("rarity", _i32), ("carity", _i32),
                ("nent", _i64), ("region", _i32), ("nrcomposed", _i32), ("nccomposed", _i32),
                ("rcomposed", _p * MAX_COMPOSED), ("ccomposed", _p * MAX_COMPOSED),
                ("roffset", _pi32), ("coffset", _pi32),
                ("roffset_quotient", _pi32), ("coffset_quotient", _pi32)]


class SparsityDesc(ctypes.Structure):
    _fields_ = [("nrows", _i64), ("ncols", _i64), ("set_diag", _i32), ("extruded", _i32),
                ("constant_layers", _i32), ("extruded_periodic", _i32), ("layers", _p),
                ("layer_slots", _i32), ("npairs", _i32), ("pairs", ctypes.POINTER(SparsityPair))]


class BCSR(ctypes.Structure):
    _fields_ = [("nrows", _i64), ("ncols", _i64), ("rdim", _i32), ("cdim", _i32),
                ("rowptr", _p), ("colidx", _p), ("values", _p)]


# name -> (restype, argtypes); the complete list of symbols include/op2g.h declares.
SIGNATURES = {
    "op2g_last_error": (ctypes.c_char_p, []),
    "op2g_abi_version": (_i32, []),
    "op2g_device_init": (_i32, [_i32, _pi32, _pi32, _pi32]),
    "op2g_kernel_create": (_i32, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(LoopDesc),
                                  ctypes.POINTER(ArgDesc), _i32, ctypes.POINTER(MapDesc), _i32,
                                  ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_p)]),
    "op2g_kernel_destroy": (None, [_p]),
    "op2g_kernel_source": (_i32, [_p, ctypes.c_char_p, ctypes.c_size_t,
                                  ctypes.POINTER(ctypes.c_size_t)]),
    "op2g_kernel_prepare": (_i32, [_p]),
    "op2g_kernel_num_ptrs": (_i32, [_p]),
    "op2g_kernel_num_regs": (_i32, [_p]),
    "op2g_kernel_launch": (_i32, [_p, ctypes.POINTER(LaunchDesc), _p]),
    "op2g_launch_shape": (None, [_i64, _i64, _i32, _i32, _i32, _i32, _i32, _pi32, _pi32, _pi32]),
    "op2g_kernel_param_bytes": (_i32, [_p]),
    "op2g_kernel_pack_params": (_i32, [_p, ctypes.POINTER(LaunchDesc), _p]),
    "op2g_kernel_launch_batched": (_i32, [_p, _p, _p, _i64, _i32, _p]),
    "op2g_graph_begin": (_i32, [ctypes.POINTER(_p)]),
    "op2g_graph_end": (_i32, [_p, ctypes.POINTER(_p)]),
    "op2g_graph_launch": (_i32, [_p, _p]),
    "op2g_graph_destroy": (None, [_p]),
    "op2g_sparsity_workspace": (_i32, [ctypes.POINTER(SparsityDesc),
                                       ctypes.POINTER(ctypes.c_size_t)]),
    "op2g_sparsity_count": (_i32, [ctypes.POINTER(SparsityDesc), _p, ctypes.c_size_t, _p,
                                   ctypes.POINTER(_i64), _p]),
    "op2g_sparsity_fill": (_i32, [ctypes.POINTER(SparsityDesc), _p, ctypes.c_size_t, _p, _p, _p]),
    "op2g_mat_zero_rows": (_i32, [ctypes.POINTER(BCSR), _p, _i64, ctypes.c_double, _p]),
    "op2g_mat_set_diagonal": (_i32, [ctypes.POINTER(BCSR), _p, _i64, ctypes.c_double, _p, _p]),
    "op2g_mat_spmv": (_i32, [ctypes.POINTER(BCSR), _p, _p, _i32, _p]),
    "op2g_colour_workspace": (_i32, [_i64, _i32, ctypes.POINTER(_i64),
                                     ctypes.POINTER(ctypes.c_size_t)]),
    "op2g_colour": (_i32, [_i64, _i32, ctypes.POINTER(_p), _pi32, ctypes.POINTER(_i64), _i32,
                           _p, ctypes.c_size_t, _p, _p, _p, _pi32, _p]),
    "op2g_colour_noalloc": (_i32, [_i64, _i32, ctypes.POINTER(_p), _pi32, ctypes.POINTER(_i64),
                                   _i32, _p, _p, _p, _pi32, _p]),
    "op2g_probe_fp64_peak": (_i32, [ctypes.POINTER(ctypes.c_double), _p]),
    "op2g_stage_plan_workspace": (_i32, [_i64, _i32, _i64, ctypes.POINTER(ctypes.c_size_t)]),
    "op2g_stage_plan_count": (_i32, [_i64, _i32, _p, _i64, _p, ctypes.c_size_t, _p, _p,
                                     ctypes.POINTER(_i64), _pi32, _p]),
    "op2g_stage_plan_fill": (_i32, [_i64, _i32, _p, _i64, _p, _p, _p, _p, _p]),
}

_lib = None


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(
                "pyop2_gb300: native library %s is missing; build it with "
                "`python -m pyop2_gb300.csrc.build`" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        if L.op2g_abi_version() != ABI_VERSION:
            raise RuntimeError("pyop2_gb300: libop2g ABI version mismatch")
        _lib = L
    return _lib


class Op2gError(RuntimeError):
    """A libop2g call failed."""

    def __init__(self, status, msg):
        super().__init__("libop2g error %d: %s" % (status, msg))
        self.status = status


def check(status):
    """Raise for a non-zero op2g_status, mapping codes to the reference's exceptions."""
    if status == OK:
        return
    msg = lib().op2g_last_error().decode(errors="replace")
    if status == ERR_COMPILE:
        raise CompilationError(msg)
    raise Op2gError(status, msg)


def call(name, *args):
    check(getattr(lib(), name)(*args))
