"""Build recipe of libop2g.so, the native engine of pyop2_gb300.

Compiles the CUDA/C++ sources of this directory with nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and links them
in-tree as ``pyop2_gb300/libop2g.so`` against the static CUDA runtime and the
NVRTC shared library.  ``op2g_device.cuh`` is embedded into the library as a
string so that NVRTC can include it when compiling par_loop wrappers.

Run as ``python -m pyop2_gb300.csrc.build`` or through ``build()``.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
ROOT = os.path.dirname(PKG)
OUT = os.path.join(PKG, "libop2g.so")
BUILD_DIR = os.path.join(HERE, "_build")

SOURCES = ["op2g_runtime.cpp", "op2g_codegen.cpp", "op2g_kernels.cu", "op2g_stage.cu"]
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _cuda_home():
    home = os.environ.get("CUDA_HOME") or os.environ.get("CUDA_PATH")
    if home and os.path.isdir(home):
        return home
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(os.path.realpath(nvcc)))
    return "/usr/local/cuda"


def _embed_header(dst):
    with open(os.path.join(HERE, "op2g_device.cuh")) as f:
        text = f.read()
    delim = "OP2G_HDR"
    assert (")" + delim + '"') not in text
    src = ('// generated by build.py from op2g_device.cuh\n'
           'namespace op2g {\n'
           'extern const char *const device_header_src;\n'
           'const char *const device_header_src = R"%s(%s)%s";\n'
           '}\n' % (delim, text, delim))
    old = None
    if os.path.exists(dst):
        with open(dst) as f:
            old = f.read()
    if old != src:
        with open(dst, "w") as f:
            f.write(src)


def _needs(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, force=False):
    """Compile libop2g.so if any source is newer than it.  Returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    if not os.path.exists(nvcc):
        nvcc = shutil.which("nvcc") or nvcc
    gen = os.path.join(BUILD_DIR, "op2g_device_src.cpp")
    _embed_header(gen)
    headers = [os.path.join(HERE, h) for h in ("op2g_internal.h", "op2g_device.cuh")]
    headers.append(os.path.join(ROOT, "include", "op2g.h"))
    jobs = []
    objs = []
    for s in SOURCES + [gen]:
        src = s if os.path.isabs(s) else os.path.join(HERE, s)
        obj = os.path.join(BUILD_DIR, os.path.basename(src) + ".o")
        objs.append(obj)
        if force or _needs(obj, [src] + headers):
            cmd = [nvcc, *ARCH_FLAGS, "-lineinfo", "-O3", "-std=c++17",
                   "-Xcompiler", "-fPIC,-O2", "-I", os.path.join(ROOT, "include"),
                   "-c", src, "-o", obj]
            if src.endswith(".cu"):
                cmd[1:1] = ["-Xptxas", "-v"] if verbose else []
            jobs.append(cmd)

    def run(cmd):
        p = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, p

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        for cmd, p in ex.map(run, jobs):
            if verbose and (p.stdout or p.stderr):
                sys.stderr.write(p.stdout + p.stderr)
            if p.returncode != 0:
                raise RuntimeError("nvcc failed:\n%s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
    if force or _needs(OUT, objs):
        libdir = os.path.join(cuda, "lib64")
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", OUT + ".tmp", *objs,
               "-L", libdir, "-lnvrtc", "-Xlinker", "-rpath," + libdir]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s%s" % (" ".join(cmd), p.stdout, p.stderr))
        os.replace(OUT + ".tmp", OUT)
    return OUT


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
