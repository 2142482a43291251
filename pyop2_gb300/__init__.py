"""pyop2_gb300: PyOP2's indirect par_loop path, native on NVIDIA GB300 (sm_103a).

The Python API mirrors ``pyop2.op2``; the work runs in libop2g.so (hand-written
CUDA + NVRTC-compiled wrappers around the user's C kernels).
"""
__version__ = "0.1.0"
