"""The C ABI of libop2g on CPU: the library loads without a GPU, exports every
symbol include/op2g.h declares, and the ctypes structures match the C layout
(checked against gcc's sizeof/offsetof of the header itself)."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "op2g.h")


@pytest.fixture(scope="module")
def lib():
    from pyop2_gb300.csrc import build
    build.build()
    from pyop2_gb300 import _lib
    return _lib


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(op2g_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_bound_functions(lib):
    assert declared_functions() == sorted(lib.SIGNATURES)


def test_library_exports_every_declared_symbol(lib):
    L = lib.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert L.op2g_abi_version() == lib.ABI_VERSION == 4
    assert L.op2g_last_error() is not None


STRUCTS = {
    "op2g_map_desc": ("MapDesc", ["kind", "arity", "base", "ncomposed", "composed", "offset",
                                  "offset_quotient", "permutation"]),
    "op2g_arg_desc": ("ArgDesc", ["kind", "access", "dtype", "dim", "map", "cmap", "rdim", "cdim",
                                  "group", "group_cols", "stride"]),
    "op2g_loop_desc": ("LoopDesc", ["extruded", "constant_layers", "extruded_periodic", "indexed",
                                    "iteration_region", "pass_layer_arg", "scatter",
                                    "block_size", "debug_checks", "batched", "prefetch",
                                    "nc_reads", "cells_per_thread"]),
    "op2g_launch_desc": ("LaunchDesc", ["start", "end", "layers", "indices", "err", "ptrs",
                                        "map_toset", "layers_per_entity", "grid", "stage"]),
    "op2g_stage_desc": ("StageDesc", ["block", "n", "ind_map", "ind_off", "ind_num", "run_off",
                                      "loc_map", "max_unique"]),
    "op2g_sparsity_pair": ("SparsityPair", ["rmap", "cmap", "rarity", "carity", "nent", "region",
                                            "nrcomposed", "nccomposed", "rcomposed", "ccomposed",
                                            "roffset", "coffset", "roffset_quotient",
                                            "coffset_quotient"]),
    "op2g_sparsity_desc": ("SparsityDesc", ["nrows", "ncols", "set_diag", "extruded",
                                            "constant_layers", "extruded_periodic", "layers",
                                            "layer_slots", "npairs", "pairs"]),
    "op2g_bcsr": ("BCSR", ["nrows", "ncols", "rdim", "cdim", "rowptr", "colidx", "values"]),
}


def test_ctypes_layout_matches_header(lib, tmp_path):
    src = ['#include <stdio.h>', '#include <stddef.h>', '#include "op2g.h"', 'int main(void) {']
    for cname, (_, fields) in STRUCTS.items():
        src.append('printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f in fields:
            src.append('printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    src.append("return 0; }")
    c = tmp_path / "layout.c"
    c.write_text("\n".join(src))
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(c), "-o", str(exe)], check=True)
    out = dict(line.rsplit(" ", 1) for line in subprocess.check_output([str(exe)]).decode().split("\n")
               if line)
    for cname, (pyname, fields) in STRUCTS.items():
        st = getattr(lib, pyname)
        assert ctypes.sizeof(st) == int(out[cname]), cname
        for f in fields:
            assert getattr(st, f).offset == int(out["%s.%s" % (cname, f)]), (cname, f)


def test_invalid_descriptor_is_rejected(lib):
    L = lib.lib()
    h = ctypes.c_void_p()
    loop = lib.LoopDesc(block_size=100)
    st = L.op2g_kernel_create(b"static void k(double *x) {}", b"k", ctypes.byref(loop), None, 0,
                              None, 0, b"sm_103a", None, ctypes.byref(h))
    assert st == lib.ERR_INVALID
    assert b"block_size" in L.op2g_last_error()


def test_graph_entry_points_reject_null(lib):
    """The graph calls validate their arguments before touching CUDA."""
    L = lib.lib()
    assert L.op2g_graph_begin(None) == lib.ERR_INVALID
    assert L.op2g_graph_end(None, None) == lib.ERR_INVALID
    assert L.op2g_graph_launch(None, None) == lib.ERR_INVALID
    L.op2g_graph_destroy(None)


def test_launch_shape_policy(lib):
    """The launch shape op2g_kernel_launch picks (a pure host function):
    threads cover every iteration, CTAs are whole warps no larger than the
    compiled size, launches of fewer than 4 full CTAs per SM run the
    balanced entry with k CTAs per SM (never for wrappers without it, never
    against an explicit grid), larger ones are capped at 4 resident waves."""
    import ctypes
    import numpy as np
    L = lib.lib()
    g, b, c = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()

    def shape(items, ents, bs, sms=152, occ=5, req=0, avail=1):
        L.op2g_launch_shape(items, ents, bs, sms, occ, req, avail, ctypes.byref(g),
                            ctypes.byref(b), ctypes.byref(c))
        return g.value, b.value, c.value

    assert shape(8192, 8192, 256) == (152, 64, 1)            # small: every SM, one warp pair
    assert shape(8192, 8192, 256, avail=0) == (32, 256, 0)   # shared staging: compiled size
    assert shape(8192, 8192, 256, req=3) == (3, 256, 0)      # explicit grid
    big = 12_582_912
    assert shape(big, big, 256) == (5 * 152 * 4, 256, 0)     # 4 resident waves
    assert shape(big, big, 256, req=-1) == ((big + 255) // 256, 256, 0)
    rng = np.random.default_rng(0)
    for _ in range(2000):
        bs = int(rng.choice([64, 128, 256, 512]))
        ents = int(rng.integers(1, 400_000))
        per = int(rng.choice([1, 1, 1, 4, 64]))
        items = ents * per
        sms = int(rng.integers(1, 200))
        gg, bb, cc = shape(items, ents, bs, sms=sms, occ=int(rng.integers(1, 9)))
        assert bb % 32 == 0 and 32 <= bb <= bs and gg >= 1
        if cc:
            assert items < 4 * sms * bs and gg <= ents
            assert gg % sms == 0 or gg == ents                 # k CTAs on every SM
            chunk = -(-ents // gg)
            assert chunk * gg >= ents                          # every entity in a chunk
        else:
            assert items >= 4 * sms * bs
