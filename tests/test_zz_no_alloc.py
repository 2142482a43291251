"""op2g_colour_noalloc: the colouring entry point for callers that cannot
allocate device memory (their device memory belongs to another allocator or a
fixed pool, or they run inside a CUDA graph capture).  It must give exactly
what op2g_colour gives with a caller-allocated workspace, call after call,
although its scratch is one fixed device array shared by all calls.

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(entry, lib, dev, maps_dev, arity, ncells, nverts, work=None):
    import torch
    colour = torch.full((ncells,), -7, dtype=torch.int32, device=dev)
    order = torch.full((ncells,), -7, dtype=torch.int32, device=dev)
    cptr = torch.full((257,), -7, dtype=torch.int64, device=dev)
    nc = ctypes.c_int32(-1)
    maps = (ctypes.c_void_p * 1)(maps_dev.data_ptr())
    ar = (ctypes.c_int32 * 1)(arity)
    tsz = (ctypes.c_int64 * 1)(nverts)
    stream = torch.cuda.current_stream().cuda_stream
    if entry == "op2g_colour":
        lib.call("op2g_colour", ncells, 1, maps, ar, tsz, 256, work.data_ptr(), work.numel(),
                 colour.data_ptr(), order.data_ptr(), cptr.data_ptr(), ctypes.byref(nc), stream)
    else:
        lib.call("op2g_colour_noalloc", ncells, 1, maps, ar, tsz, 256, colour.data_ptr(),
                 order.data_ptr(), cptr.data_ptr(), ctypes.byref(nc), stream)
    torch.cuda.synchronize()
    return colour.cpu().numpy(), order.cpu().numpy(), cptr.cpu().numpy(), nc.value


def test_noalloc_colouring_matches_workspace_colouring(gpu_op2):
    import torch
    from pyop2_gb300 import _lib, device, meshes
    dev = device.device()
    coords, cells = meshes.unit_cube_tets(12, permute=True, seed=5)   # 10,368 tets
    ncells, nverts = cells.shape[0], coords.shape[0]
    maps_dev = torch.from_numpy(cells).to(dev)
    ws = ctypes.c_size_t()
    tsz = (ctypes.c_int64 * 1)(nverts)
    _lib.call("op2g_colour_workspace", ncells, 1, tsz, ctypes.byref(ws))
    assert ws.value <= 16 * 1024 * 1024
    work = torch.empty(ws.value, dtype=torch.uint8, device=dev)
    ref = _run("op2g_colour", _lib, dev, maps_dev, 4, ncells, nverts, work)
    assert ref[3] > 1
    for _ in range(2):   # the shared scratch keeps the previous call's contents
        got = _run("op2g_colour_noalloc", _lib, dev, maps_dev, 4, ncells, nverts)
        assert got[3] == ref[3]
        np.testing.assert_array_equal(got[0], ref[0])
        np.testing.assert_array_equal(got[1], ref[1])
        np.testing.assert_array_equal(got[2], ref[2])
    # and the colouring is valid: no two cells of one colour share a vertex
    colour, order, cptr, nc = got
    for c in range(nc):
        seg = order[cptr[c]:cptr[c + 1]]
        assert np.all(colour[seg] == c)
        v = cells[seg].ravel()
        assert len(np.unique(v)) == len(v)


def test_noalloc_colouring_rejects_oversized_problems(gpu_op2):
    from pyop2_gb300 import _lib
    L = _lib.lib()
    tsz = (ctypes.c_int64 * 1)(10_000_000)     # 400 MB of target state > 16 MiB
    maps = (ctypes.c_void_p * 1)(None)
    ar = (ctypes.c_int32 * 1)(4)
    nc = ctypes.c_int32()
    st = L.op2g_colour_noalloc(1000, 1, maps, ar, tsz, 256, None, None, None, ctypes.byref(nc),
                               None)
    assert st == _lib.ERR_CAPACITY
    assert b"scratch" in L.op2g_last_error()
