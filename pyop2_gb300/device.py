"""Device memory and host mirrors.

Every Dat, Global, Map and Mat keeps its data in HBM as a torch CUDA tensor
(torch is only the allocator and stream provider here) with a lazily
materialised host mirror, following the device-state protocol of the
historical OP2 CUDA backend (doc/sphinx/source/backends.rst:222-236): the host
copy is refreshed only when the host reads data that the device modified, and
uploaded only when a launch needs data that the host modified.
"""
import warnings

import numpy as np
import torch

from pyop2_gb300 import _lib
from pyop2_gb300.configuration import configuration

_ready = False
_sm_count = 0
_cc = (0, 0)


def available():
    """True if a CUDA device can be used."""
    return torch.cuda.is_available()


def require():
    """Initialise libop2g on the configured device; fail loudly without one."""
    global _ready, _sm_count, _cc
    if _ready:
        return
    if not torch.cuda.is_available():
        raise RuntimeError("pyop2_gb300 executes par_loops on a CUDA device and none is "
                           "available (there is no CPU fallback)")
    dev = configuration["device"]
    torch.cuda.set_device(dev)
    sm = _lib.ctypes.c_int32()
    ma = _lib.ctypes.c_int32()
    mi = _lib.ctypes.c_int32()
    _lib.call("op2g_device_init", dev, _lib.ctypes.byref(sm), _lib.ctypes.byref(ma),
              _lib.ctypes.byref(mi))
    _sm_count = sm.value
    _cc = (ma.value, mi.value)
    _ready = True


def device():
    require()
    return torch.device("cuda", configuration["device"])


def sm_count():
    require()
    return _sm_count


_raw_stream = getattr(torch._C, "_cuda_getCurrentRawStream", None)
_get_device = getattr(torch._C, "_cuda_getDevice", None)


def stream_handle():
    """cudaStream_t of torch's current stream on the current device, as an int
    for ctypes (through torch's direct accessors when present: the public
    torch.cuda.current_stream() costs several microseconds per call)."""
    if _raw_stream is not None and _get_device is not None:
        return _raw_stream(_get_device())
    return torch.cuda.current_stream().cuda_stream


_TORCH = {
    "float64": torch.float64, "float32": torch.float32, "int32": torch.int32,
    "int64": torch.int64, "int16": torch.int16, "int8": torch.int8, "uint8": torch.uint8,
}
if hasattr(torch, "uint32"):
    _TORCH["uint32"] = torch.uint32
    _TORCH["uint64"] = torch.uint64
if hasattr(torch, "uint16"):
    _TORCH["uint16"] = torch.uint16


def torch_dtype(dtype):
    return _TORCH[np.dtype(dtype).name]


def empty_bytes(nbytes):
    """Uninitialised device buffer of nbytes (at least 1) as a uint8 tensor."""
    return torch.empty(max(int(nbytes), 1), dtype=torch.uint8, device=device())


def zeros_bytes(nbytes):
    return torch.zeros(max(int(nbytes), 1), dtype=torch.uint8, device=device())


def upload(arr, out=None):
    """Copy a host array into a (new or given) device byte buffer."""
    a = np.ascontiguousarray(arr)
    src = None
    if a.size:
        with warnings.catch_warnings():
            # read-only host arrays (Map values) are only read by the copy
            warnings.simplefilter("ignore", UserWarning)
            src = torch.from_numpy(a.reshape(-1).view(np.uint8))
    if out is None:
        out = empty_bytes(a.nbytes)
    if src is not None:
        out[:a.nbytes].copy_(src, non_blocking=False)
    return out


def download(buf, dtype, shape, out=None):
    """Copy a device byte buffer into a host array of dtype/shape."""
    dtype = np.dtype(dtype)
    n = int(np.prod(shape)) * dtype.itemsize
    if out is None:
        out = np.empty(shape, dtype=dtype)
    if n:
        dst = torch.from_numpy(out.reshape(-1).view(np.uint8))
        dst.copy_(buf[:n])
    return out


def ptr(t):
    """Device address of a tensor (0 for None)."""
    return 0 if t is None else t.data_ptr()


class Mirror:
    """A host array with a device twin.

    state: "host" (host newer), "device" (device newer) or "both".  The host
    array is allocated lazily; a never-touched buffer is zero on both sides.
    """

    def __init__(self, dtype, shape, data=None):
        self.dtype = np.dtype(dtype)
        self.shape = tuple(shape)
        self._host = data           # numpy array or None (= zeros)
        self._dev = None            # torch uint8 tensor or None
        self.state = "host"

    @property
    def nbytes(self):
        return int(np.prod(self.shape)) * self.dtype.itemsize

    # ---- host side
    def host(self, write):
        """Host array, made current; `write` marks the host as newer."""
        if self._host is None:
            if self._dev is not None and self.state == "device":
                self._host = download(self._dev, self.dtype, self.shape)
            else:
                self._host = np.zeros(self.shape, dtype=self.dtype)
        elif self.state == "device":
            download(self._dev, self.dtype, self.shape, out=self._host)
        if self._dev is not None:
            self.state = "host" if write else "both"
        else:
            self.state = "host"
        return self._host

    def host_allocated(self):
        return self._host is not None

    # ---- device side
    def dev(self):
        """Device buffer holding the current data."""
        if self._dev is None:
            if self._host is None:
                self._dev = zeros_bytes(self.nbytes)
            else:
                self._dev = upload(self._host)
            self.state = "both" if self._host is not None else "device"
        elif self.state == "host":
            upload(self._host, out=self._dev)
            self.state = "both"
        return self._dev

    def dev_modified(self):
        """Call after a launch wrote the device buffer."""
        self.state = "device"

    def tensor(self):
        """Typed device view (shape-flattened) of the current data."""
        b = self.dev()
        n = self.nbytes
        return b[:n].view(torch_dtype(self.dtype)) if n else \
            torch.empty(0, dtype=torch_dtype(self.dtype), device=b.device)

    def zero(self):
        if self._dev is not None:
            # the host copy goes stale (refreshed if it is read) instead of
            # being cleared as well
            self._dev.zero_()
            self.state = "device"
        else:
            self._host = None
            self.state = "host"
