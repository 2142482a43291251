"""op2g_colour_noalloc: the colouring entry point for callers that cannot
allocate device memory (their device memory belongs to another allocator or a
pool sized up front, or their runtime forbids cudaMalloc after start-up).  It
must give exactly what op2g_colour gives with a caller-allocated workspace,
call after call, although its scratch is one fixed device array shared by all
calls and left holding whatever the previous call wrote.

This file is named to be collected last, so a run that stops at the first
failure has run every other test before it."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(entry, lib, dev, maps_dev, arity, ncells, nverts, work=None):
    """One colouring through the C ABI; maps_dev, arity and nverts may be
    lists (one entry per map)."""
    import torch
    if not isinstance(maps_dev, (list, tuple)):
        maps_dev, arity, nverts = [maps_dev], [arity], [nverts]
    nm = len(maps_dev)
    colour = torch.full((max(ncells, 1),), -7, dtype=torch.int32, device=dev)
    order = torch.full((max(ncells, 1),), -7, dtype=torch.int32, device=dev)
    cptr = torch.full((257,), -7, dtype=torch.int64, device=dev)
    nc = ctypes.c_int32(-1)
    maps = (ctypes.c_void_p * nm)(*[m.data_ptr() for m in maps_dev])
    ar = (ctypes.c_int32 * nm)(*arity)
    tsz = (ctypes.c_int64 * nm)(*nverts)
    stream = torch.cuda.current_stream().cuda_stream
    if entry == "op2g_colour":
        lib.call("op2g_colour", ncells, nm, maps, ar, tsz, 256, work.data_ptr(), work.numel(),
                 colour.data_ptr(), order.data_ptr(), cptr.data_ptr(), ctypes.byref(nc), stream)
    else:
        lib.call("op2g_colour_noalloc", ncells, nm, maps, ar, tsz, 256, colour.data_ptr(),
                 order.data_ptr(), cptr.data_ptr(), ctypes.byref(nc), stream)
    torch.cuda.synchronize()
    return (colour.cpu().numpy()[:ncells], order.cpu().numpy()[:ncells], cptr.cpu().numpy(),
            nc.value)


def _workspace(lib, dev, ncells, nverts):
    import torch
    nverts = nverts if isinstance(nverts, (list, tuple)) else [nverts]
    ws = ctypes.c_size_t()
    tsz = (ctypes.c_int64 * len(nverts))(*nverts)
    lib.call("op2g_colour_workspace", ncells, len(nverts), tsz, ctypes.byref(ws))
    assert ws.value <= 16 * 1024 * 1024
    return torch.empty(ws.value, dtype=torch.uint8, device=dev)


def test_noalloc_colouring_matches_workspace_colouring(gpu_op2):
    import torch
    from pyop2_gb300 import _lib, device, meshes
    dev = device.device()
    coords, cells = meshes.unit_cube_tets(12, permute=True, seed=5)   # 10,368 tets
    ncells, nverts = cells.shape[0], coords.shape[0]
    maps_dev = torch.from_numpy(cells).to(dev)
    ref = _run("op2g_colour", _lib, dev, maps_dev, 4, ncells, nverts,
               _workspace(_lib, dev, ncells, nverts))
    assert ref[3] > 1
    # a larger two-map problem, run between the checked calls, leaves non-zero
    # bytes at other offsets of the shared scratch (target states, histogram)
    c2, cells2 = meshes.unit_cube_tets(16, permute=True, seed=6)     # 24,576 tets
    v2 = c2.shape[0]
    edges = np.stack([cells2[:, 0], cells2[:, 3]], axis=1).astype(np.int32)
    big = [torch.from_numpy(cells2).to(dev), torch.from_numpy(edges).to(dev)]
    for i in range(2):   # the shared scratch keeps the previous call's contents
        got = _run("op2g_colour_noalloc", _lib, dev, maps_dev, 4, ncells, nverts)
        assert got[3] == ref[3]
        np.testing.assert_array_equal(got[0], ref[0])
        np.testing.assert_array_equal(got[1], ref[1])
        np.testing.assert_array_equal(got[2], ref[2])
        if i == 0:
            other = _run("op2g_colour_noalloc", _lib, dev, big, [4, 2], cells2.shape[0],
                         [v2, v2])
            other_ref = _run("op2g_colour", _lib, dev, big, [4, 2], cells2.shape[0], [v2, v2],
                             _workspace(_lib, dev, cells2.shape[0], [v2, v2]))
            np.testing.assert_array_equal(other[0], other_ref[0])
    # and the colouring is valid: no two cells of one colour share a vertex
    colour, order, cptr, nc = got
    for c in range(nc):
        seg = order[cptr[c]:cptr[c + 1]]
        assert np.all(colour[seg] == c)
        v = cells[seg].ravel()
        assert len(np.unique(v)) == len(v)


def test_empty_iteration_set(gpu_op2):
    """No entities: no colours, a zero colour_ptr, nothing written past the
    workspace, from both entry points."""
    import torch
    from pyop2_gb300 import _lib, device
    dev = device.device()
    m = torch.zeros(4, dtype=torch.int32, device=dev)
    work = _workspace(_lib, dev, 0, 10)
    guard = torch.full((4096,), 0x5A, dtype=torch.uint8, device=dev)
    pad = torch.cat([work, guard])
    ref = _run("op2g_colour", _lib, dev, m, 4, 0, 10, pad[:work.numel()])
    assert ref[3] == 0 and not np.any(ref[2])
    assert bool((pad[work.numel():] == 0x5A).all())
    got = _run("op2g_colour_noalloc", _lib, dev, m, 4, 0, 10)
    assert got[3] == 0 and not np.any(got[2])


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
