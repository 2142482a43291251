// op2g_runtime.cpp -- C ABI of the par_loop engine: NVRTC compilation of the
// generated wrappers, an on-disk cubin cache, module loading and launches.
//
// Replaces the reference's JIT pipeline (pyop2/compilation.py:427-626: write
// C, run gcc, cache the .so, ctypes.CDLL) and the ctypes call of the wrapper
// (pyop2/global_kernel.py:322-331).  Driver-API entry points are fetched
// through the CUDA runtime (cudaGetDriverEntryPointByVersion), so the library
// loads on machines without a GPU driver and only needs one when a kernel is
// launched.
#include <cuda.h>
#include <cuda_runtime_api.h>
#include <nvrtc.h>

#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <sys/stat.h>
#include <unistd.h>

#include "op2g_internal.h"

namespace op2g {

static thread_local std::string g_last_error = "no error";

op2g_status fail(op2g_status code, const std::string &msg) {
    g_last_error = msg;
    return code;
}

op2g_status cuda_fail(int err, const char *what) {
    std::ostringstream s;
    s << what << ": " << cudaGetErrorName((cudaError_t)err) << " ("
      << cudaGetErrorString((cudaError_t)err) << ")";
    return fail(OP2G_ERR_CUDA, s.str());
}

// ------------------------------------------------------------ driver API
struct Driver {
    CUresult (*ModuleLoadData)(CUmodule *, const void *) = nullptr;
    CUresult (*ModuleUnload)(CUmodule) = nullptr;
    CUresult (*ModuleGetFunction)(CUfunction *, CUmodule, const char *) = nullptr;
    CUresult (*LaunchKernel)(CUfunction, unsigned, unsigned, unsigned, unsigned, unsigned,
                             unsigned, unsigned, CUstream, void **, void **) = nullptr;
    CUresult (*FuncGetAttribute)(int *, CUfunction_attribute, CUfunction) = nullptr;
    CUresult (*OccupancyMaxActiveBlocksPerMultiprocessor)(int *, CUfunction, int,
                                                          size_t) = nullptr;
    CUresult (*FuncSetAttribute)(CUfunction, CUfunction_attribute, int) = nullptr;
    CUresult (*GetErrorString)(CUresult, const char **) = nullptr;
    bool ok = false;
    std::string why;
};

static Driver &driver() {
    static Driver d;
    static std::once_flag once;
    std::call_once(once, [] {
        struct Sym {
            const char *name;
            void **slot;
        } syms[] = {
            {"cuModuleLoadData", (void **)&d.ModuleLoadData},
            {"cuModuleUnload", (void **)&d.ModuleUnload},
            {"cuModuleGetFunction", (void **)&d.ModuleGetFunction},
            {"cuLaunchKernel", (void **)&d.LaunchKernel},
            {"cuFuncGetAttribute", (void **)&d.FuncGetAttribute},
            {"cuOccupancyMaxActiveBlocksPerMultiprocessor",
             (void **)&d.OccupancyMaxActiveBlocksPerMultiprocessor},
            {"cuGetErrorString", (void **)&d.GetErrorString},
            {"cuFuncSetAttribute", (void **)&d.FuncSetAttribute},
        };
        for (auto &s : syms) {
            cudaDriverEntryPointQueryResult q;
            cudaError_t e = cudaGetDriverEntryPointByVersion(s.name, s.slot, 12000,
                                                             cudaEnableDefault, &q);
            if (e != cudaSuccess || q != cudaDriverEntryPointSuccess || !*s.slot) {
                d.why = std::string("driver entry point ") + s.name + " unavailable (" +
                        cudaGetErrorString(e) + ")";
                return;
            }
        }
        d.ok = true;
    });
    return d;
}

static op2g_status cu_fail(CUresult r, const char *what) {
    const char *s = "unknown";
    if (driver().GetErrorString) driver().GetErrorString(r, &s);
    return fail(OP2G_ERR_CUDA, std::string(what) + ": CUDA driver error " + std::to_string((int)r) +
                                   " (" + (s ? s : "") + ")");
}

// -------------------------------------------------------------- hashing
static void fnv1a(const std::string &s, uint64_t &h) {
    for (unsigned char c : s) {
        h ^= c;
        h *= 1099511628211ull;
    }
}
static std::string hash_hex(const std::string &s) {
    uint64_t a = 1469598103934665603ull, b = 0x9e3779b97f4a7c15ull;
    fnv1a(s, a);
    fnv1a(std::to_string(s.size()) + s, b);
    char buf[40];
    snprintf(buf, sizeof buf, "%016llx%016llx", (unsigned long long)a, (unsigned long long)b);
    return buf;
}

static bool read_file(const std::string &path, std::string &out) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return false;
    std::string buf;
    char tmp[1 << 16];
    size_t n;
    while ((n = fread(tmp, 1, sizeof tmp, f)) > 0) buf.append(tmp, n);
    fclose(f);
    out.swap(buf);
    return true;
}

static void mkdirs(const std::string &dir) {
    std::string cur;
    for (size_t i = 0; i < dir.size(); ++i) {
        cur.push_back(dir[i]);
        if (dir[i] == '/' || i + 1 == dir.size()) mkdir(cur.c_str(), 0755);
    }
}

static void write_file_atomic(const std::string &path, const std::string &data) {
    std::string tmp = path + ".tmp." + std::to_string((long long)getpid());
    FILE *f = fopen(tmp.c_str(), "wb");
    if (!f) return;
    bool ok = fwrite(data.data(), 1, data.size(), f) == data.size();
    ok = (fclose(f) == 0) && ok;
    if (ok) rename(tmp.c_str(), path.c_str());
    else unlink(tmp.c_str());
}

std::string current_arch(op2g_status *st) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    int maj = 0, min = 0;
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&maj, cudaDevAttrComputeCapabilityMajor, dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&min, cudaDevAttrComputeCapabilityMinor, dev);
    if (e != cudaSuccess) {
        *st = cuda_fail(e, "querying the current device");
        return "";
    }
    *st = OP2G_OK;
    return "sm_" + std::to_string(maj) + std::to_string(min) + (maj >= 9 ? "a" : "");
}

static op2g_status nvrtc_compile(const std::string &src, const std::string &arch,
                                 std::string &cubin) {
    nvrtcProgram prog;
    const char *hdrs[] = {device_header_src};
    const char *names[] = {"op2g_device.cuh"};
    nvrtcResult r = nvrtcCreateProgram(&prog, src.c_str(), "op2g_wrapper.cu", 1, hdrs, names);
    if (r != NVRTC_SUCCESS)
        return fail(OP2G_ERR_COMPILE, std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r));
    std::string archopt = "--gpu-architecture=" + arch;
    const char *opts[] = {archopt.c_str(), "--device-as-default-execution-space", "-std=c++17",
                          "-lineinfo", "-w"};
    r = nvrtcCompileProgram(prog, sizeof opts / sizeof opts[0], opts);
    size_t logsz = 0;
    nvrtcGetProgramLogSize(prog, &logsz);
    std::string log(logsz, '\0');
    if (logsz) nvrtcGetProgramLog(prog, &log[0]);
    while (!log.empty() && log.back() == '\0') log.pop_back();
    if (r != NVRTC_SUCCESS) {
        nvrtcDestroyProgram(&prog);
        return fail(OP2G_ERR_COMPILE, std::string("NVRTC compilation failed (") +
                                          nvrtcGetErrorString(r) + "):\n" + log +
                                          "\n---- generated source ----\n" + src);
    }
    size_t n = 0;
    r = nvrtcGetCUBINSize(prog, &n);
    if (r == NVRTC_SUCCESS) {
        cubin.resize(n);
        r = nvrtcGetCUBIN(prog, &cubin[0]);
    }
    nvrtcDestroyProgram(&prog);
    if (r != NVRTC_SUCCESS)
        return fail(OP2G_ERR_COMPILE, std::string("nvrtcGetCUBIN: ") + nvrtcGetErrorString(r));
    return OP2G_OK;
}

// Compile (or fetch from the cache dir) the cubin for `src`.
op2g_status build_cubin(const std::string &src, const std::string &arch, const char *cache_dir,
                        std::string &cubin) {
    std::string key = hash_hex(src + "\n//arch=" + arch + "\n//abi=" +
                               std::to_string(OP2G_ABI_VERSION) + "\n" + device_header_src);
    std::string path;
    if (cache_dir && *cache_dir) {
        path = std::string(cache_dir) + "/op2g-" + key + "-" + arch + ".cubin";
        if (read_file(path, cubin) && !cubin.empty()) return OP2G_OK;
    }
    op2g_status st = nvrtc_compile(src, arch, cubin);
    if (st != OP2G_OK) return st;
    if (!path.empty()) {
        mkdirs(cache_dir);
        write_file_atomic(path, cubin);
    }
    return OP2G_OK;
}

struct Loaded {
    CUmodule mod = nullptr;
    CUfunction f = nullptr, fb = nullptr, fc = nullptr;  // plain, batched, chunked
    int regs = -1;
    int occ = 0;  // resident CTAs per SM
    int sms = 0;
    // staged wrappers: dynamic shared memory the function is set up for, and
    // the resident CTAs per SM at the last size asked for
    int smem_attr = 0;
    size_t occ_smem = (size_t)-1;
    int occ_at_smem = 0;
};

// Load `cubin` on the current device (cached per device in `per_dev`).
op2g_status load_module(const std::string &cubin, const char *fname, const char *fname_b, int bs,
                        std::map<int, Loaded> &per_dev, std::mutex &mu, Loaded **out) {
    Driver &D = driver();
    if (!D.ok) return fail(OP2G_ERR_CUDA, "CUDA driver not available: " + D.why);
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
    std::lock_guard<std::mutex> g(mu);
    auto it = per_dev.find(dev);
    if (it != per_dev.end()) {
        *out = &it->second;
        return OP2G_OK;
    }
    e = cudaFree(nullptr);  // make sure the primary context is current
    if (e != cudaSuccess) return cuda_fail(e, "initialising the CUDA context");
    Loaded L;
    CUresult r = D.ModuleLoadData(&L.mod, cubin.data());
    if (r != CUDA_SUCCESS) return cu_fail(r, "cuModuleLoadData");
    r = D.ModuleGetFunction(&L.f, L.mod, fname);
    if (r != CUDA_SUCCESS) return cu_fail(r, "cuModuleGetFunction");
    if (fname_b) {
        r = D.ModuleGetFunction(&L.fb, L.mod, fname_b);
        if (r != CUDA_SUCCESS) return cu_fail(r, "cuModuleGetFunction (batched)");
    }
    // the balanced entry exists only in wrappers without shared-memory staging
    if (D.ModuleGetFunction(&L.fc, L.mod, "op2g_wrap_chunked") != CUDA_SUCCESS) L.fc = nullptr;
    D.FuncGetAttribute(&L.regs, CU_FUNC_ATTRIBUTE_NUM_REGS, L.f);
    if (D.OccupancyMaxActiveBlocksPerMultiprocessor(&L.occ, L.f, bs, 0) != CUDA_SUCCESS) L.occ = 1;
    if (L.occ < 1) L.occ = 1;
    cudaDeviceGetAttribute(&L.sms, cudaDevAttrMultiProcessorCount, dev);
    if (L.sms < 1) L.sms = 1;
    auto res = per_dev.emplace(dev, L);
    *out = &res.first->second;
    return OP2G_OK;
}

op2g_status launch(CUfunction f, unsigned grid, unsigned block, void **params, void *stream,
                   unsigned smem = 0) {
    CUresult r = driver().LaunchKernel(f, grid, 1, 1, block, 1, 1, smem, (CUstream)stream, params,
                                       nullptr);
    if (r != CUDA_SUCCESS) return cu_fail(r, "cuLaunchKernel");
    return OP2G_OK;
}

}  // namespace op2g

using namespace op2g;

// True when the wrapper spreads the layers of a column over threads (the
// codegen's choice for constant layers without written direct arguments).
static bool column_parallel(const Signature &S) {
    if (!S.loop.extruded || !S.loop.constant_layers || S.loop.scatter == OP2G_SCATTER_PLAIN)
        return false;
    for (const ArgInfo &A : S.args)
        if (A.d.kind == OP2G_ARG_DAT && A.d.map < 0 && A.d.access != OP2G_READ) return false;
    return true;
}

struct op2g_kernel {
    Signature sig;
    std::string source, arch, cubin;
    std::mutex mu;
    std::map<int, Loaded> per_dev;
    int param_bytes = 0;
    bool staged = false;   // the wrapper stages arguments on a plan (OP2G_SCATTER_STAGED)
    int cells_per_thread = 1;
    // Direct arguments with rows of a multiple of 16 bytes (pointer slot,
    // alignment): a second variant of the wrapper declares their rows
    // aligned, and a launch runs it when every such pointer is aligned.
    std::vector<std::pair<int, int>> al_args;
    std::string source_al, cubin_al;
    std::map<int, Loaded> per_dev_al;
};

// Whether the launch's direct-argument pointers allow the aligned variant.
static bool use_aligned(const op2g_kernel *k, const op2g_launch_desc *d) {
    if (k->al_args.empty() || !d->ptrs) return false;
    for (const auto &sa : k->al_args)
        if ((uintptr_t)d->ptrs[sa.first] % (uintptr_t)sa.second) return false;
    return true;
}

extern "C" {

const char *op2g_last_error(void) { return g_last_error.c_str(); }

int32_t op2g_abi_version(void) { return OP2G_ABI_VERSION; }

op2g_status op2g_device_init(int32_t device, int32_t *sm_count, int32_t *cc_major,
                             int32_t *cc_minor) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) return cuda_fail(e, "cudaSetDevice");
    e = cudaFree(nullptr);
    if (e != cudaSuccess) return cuda_fail(e, "initialising the CUDA context");
    int v = 0;
    if (sm_count) {
        cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device);
        *sm_count = v;
    }
    if (cc_major) {
        cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMajor, device);
        *cc_major = v;
    }
    if (cc_minor) {
        cudaDeviceGetAttribute(&v, cudaDevAttrComputeCapabilityMinor, device);
        *cc_minor = v;
    }
    if (!driver().ok) return fail(OP2G_ERR_CUDA, "CUDA driver not available: " + driver().why);
    return OP2G_OK;
}

op2g_status op2g_kernel_create(const char *user_src, const char *kernel_name,
                               const op2g_loop_desc *loop, const op2g_arg_desc *args,
                               int32_t nargs, const op2g_map_desc *maps, int32_t nmaps,
                               const char *arch, const char *cache_dir, op2g_kernel **out) {
    if (!out) return fail(OP2G_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!user_src || !kernel_name || !loop) return fail(OP2G_ERR_INVALID, "NULL argument");
    if (nargs < 0 || nargs > OP2G_MAX_ARGS) return fail(OP2G_ERR_INVALID, "too many arguments");
    if (nmaps < 0 || nmaps > OP2G_MAX_MAPS) return fail(OP2G_ERR_INVALID, "too many maps");
    if ((nargs && !args) || (nmaps && !maps)) return fail(OP2G_ERR_INVALID, "NULL descriptors");
    Signature S;
    S.user_src = user_src;
    S.kernel_name = kernel_name;
    S.loop = *loop;
    S.block_size = loop->block_size > 0 ? loop->block_size : 256;
    if (S.block_size % 32 || S.block_size > 1024)
        return fail(OP2G_ERR_INVALID, "block_size must be a multiple of 32 and <= 1024");
    if (loop->iteration_region < OP2G_ON_BOTTOM || loop->iteration_region > OP2G_ALL)
        S.loop.iteration_region = OP2G_ALL;
    int slot = 0;
    for (int a = 0; a < nargs; ++a) {
        ArgInfo A;
        A.d = args[a];
        A.slot = slot;
        slot += (A.d.kind == OP2G_ARG_MAT) ? 3 : 1;
        S.args.push_back(A);
    }
    S.map_slot0 = slot;
    for (int m = 0; m < nmaps; ++m) {
        MapInfo M;
        M.kind = maps[m].kind;
        M.arity = maps[m].arity;
        M.base = maps[m].base;
        M.ncomposed = maps[m].ncomposed;
        for (int k = 0; k < OP2G_MAX_COMPOSED; ++k) M.composed[k] = maps[m].composed[k];
        if (M.arity > 0 && M.arity < (1 << 20)) {
            if (maps[m].offset) M.offset.assign(maps[m].offset, maps[m].offset + M.arity);
            if (maps[m].offset_quotient)
                M.offset_quotient.assign(maps[m].offset_quotient, maps[m].offset_quotient + M.arity);
            if (maps[m].permutation)
                M.permutation.assign(maps[m].permutation, maps[m].permutation + M.arity);
        }
        S.maps.push_back(M);
    }
    S.nptrs = slot + nmaps;
    std::string why = validate_signature(S);
    if (!why.empty()) return fail(OP2G_ERR_INVALID, why);

    op2g_kernel *k = new op2g_kernel();
    k->sig = S;
    k->source = generate_source(S, &k->cells_per_thread);
    k->param_bytes = 8 * (5 + (S.nptrs > 0 ? S.nptrs : 1) + (nmaps > 0 ? nmaps : 1));
    for (int r : staged_args(S))
        if (r >= 0) k->staged = true;
    if (k->staged) k->param_bytes += 8 * (2 + 6 * (nmaps > 0 ? nmaps : 1));
    op2g_status st = OP2G_OK;
    k->arch = (arch && *arch) ? std::string(arch) : current_arch(&st);
    if (st != OP2G_OK) {
        delete k;
        return st;
    }
    st = build_cubin(k->source, k->arch, cache_dir, k->cubin);
    if (st == OP2G_OK) {
        k->al_args = aligned_direct_args(S);
        if (!k->al_args.empty()) {
            k->source_al = generate_source(S, nullptr, true);
            st = build_cubin(k->source_al, k->arch, cache_dir, k->cubin_al);
        }
    }
    if (st != OP2G_OK) {
        delete k;
        return st;
    }
    *out = k;
    return OP2G_OK;
}

void op2g_kernel_destroy(op2g_kernel *k) {
    if (!k) return;
    if (driver().ok) {
        for (auto &kv : k->per_dev)
            if (kv.second.mod) driver().ModuleUnload(kv.second.mod);
        for (auto &kv : k->per_dev_al)
            if (kv.second.mod) driver().ModuleUnload(kv.second.mod);
    }
    delete k;
}

op2g_status op2g_kernel_source(const op2g_kernel *k, char *buf, size_t len, size_t *needed) {
    if (!k) return fail(OP2G_ERR_INVALID, "NULL kernel");
    if (needed) *needed = k->source.size() + 1;
    if (buf && len) {
        size_t n = k->source.size() < len - 1 ? k->source.size() : len - 1;
        memcpy(buf, k->source.data(), n);
        buf[n] = '\0';
    }
    return OP2G_OK;
}

op2g_status op2g_kernel_prepare(op2g_kernel *k) {
    if (!k) return fail(OP2G_ERR_INVALID, "NULL kernel");
    Loaded *L = nullptr;
    op2g_status st = load_module(k->cubin, "op2g_wrap", "op2g_wrap_batched", k->sig.block_size,
                                 k->per_dev, k->mu, &L);
    if (st == OP2G_OK && !k->cubin_al.empty())
        st = load_module(k->cubin_al, "op2g_wrap", "op2g_wrap_batched", k->sig.block_size,
                         k->per_dev_al, k->mu, &L);
    return st;
}

int32_t op2g_kernel_num_ptrs(const op2g_kernel *k) { return k ? k->sig.nptrs : -1; }

int32_t op2g_kernel_num_regs(const op2g_kernel *k) {
    if (!k) return -1;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    auto it = k->per_dev.find(dev);
    return it == k->per_dev.end() ? -1 : it->second.regs;
}

int32_t op2g_kernel_param_bytes(const op2g_kernel *k) { return k ? k->param_bytes : -1; }

op2g_status op2g_kernel_pack_params(const op2g_kernel *k, const op2g_launch_desc *d, void *out) {
    if (!k || !d || !out) return fail(OP2G_ERR_INVALID, "NULL argument");
    if (!d->ptrs && k->sig.nptrs > 0) return fail(OP2G_ERR_INVALID, "ptrs is NULL");
    const Signature &S = k->sig;
    if (S.loop.extruded && !d->layers) return fail(OP2G_ERR_INVALID, "extruded loop needs layers");
    if (S.loop.indexed && !d->indices) return fail(OP2G_ERR_INVALID, "indexed loop needs indices");
    int64_t *w = (int64_t *)out;
    memset(out, 0, k->param_bytes);
    w[0] = d->start;
    w[1] = d->end;
    w[2] = (int64_t)(intptr_t)d->layers;
    w[3] = (int64_t)(intptr_t)d->indices;
    w[4] = (int64_t)(intptr_t)d->err;
    for (int i = 0; i < S.nptrs; ++i) w[5 + i] = (int64_t)(intptr_t)d->ptrs[i];
    const int np = S.nptrs > 0 ? S.nptrs : 1;
    for (size_t m = 0; m < S.maps.size(); ++m)
        w[5 + np + m] = d->map_toset ? d->map_toset[m] : INT64_MAX;
    if (k->staged) {
        // sblock, sn, smax[nm], sind[nm], soff[nm], snum[nm], sruns[nm], sloc[nm]
        const op2g_stage_desc *g = d->stage;
        if (!g || g->block <= 0) return fail(OP2G_ERR_INVALID, "staged wrapper launched without a plan");
        const int nm = S.maps.empty() ? 1 : (int)S.maps.size();
        if (d->end > g->n) return fail(OP2G_ERR_INVALID, "launch range beyond the staging plan");
        int64_t *x = w + 5 + np + nm + 1;
        x[-1] = g->block;
        x[0] = g->n;
        std::vector<int> st = staged_args(S);
        for (size_t a = 0; a < st.size(); ++a) {
            const int m = st[a];
            if (m < 0) continue;
            if (!g->ind_map[m] || !g->ind_off[m] || !g->ind_num[m] || !g->run_off[m] ||
                !g->loc_map[m] || g->max_unique[m] < 0)
                return fail(OP2G_ERR_INVALID, "staging plan lacks map " + std::to_string(m));
            if (g->block * S.maps[m].arity > 65535)
                return fail(OP2G_ERR_INVALID, "staging plan partitions are too large");
            if ((uintptr_t)g->loc_map[m] % 8)
                return fail(OP2G_ERR_INVALID, "loc_map array is not 8-byte aligned");
        }
        for (int m = 0; m < (int)S.maps.size(); ++m) {
            x[1 + m] = g->max_unique[m];
            x[1 + nm + m] = (int64_t)(intptr_t)g->ind_map[m];
            x[1 + 2 * nm + m] = (int64_t)(intptr_t)g->ind_off[m];
            x[1 + 3 * nm + m] = (int64_t)(intptr_t)g->ind_num[m];
            x[1 + 4 * nm + m] = (int64_t)(intptr_t)g->run_off[m];
            x[1 + 5 * nm + m] = (int64_t)(intptr_t)g->loc_map[m];
        }
    }
    // Every slot the generated code dereferences must be non-NULL.
    for (const ArgInfo &A : S.args) {
        int nslots = A.d.kind == OP2G_ARG_MAT ? 3 : 1;
        for (int s = 0; s < nslots; ++s)
            if (!d->ptrs[A.slot + s] && A.d.kind != OP2G_ARG_PASSTHROUGH)
                return fail(OP2G_ERR_INVALID, "NULL device pointer for an argument");
    }
    for (size_t m = 0; m < S.maps.size(); ++m) {
        if (S.maps[m].kind != OP2G_MAP_PLAIN) continue;
        const void *mp = d->ptrs[S.map_slot((int)m)];
        if (!mp) return fail(OP2G_ERR_INVALID, "NULL device pointer for map " + std::to_string(m));
        // rows are read as int4 / int2 vectors
        const int ar = S.maps[m].arity;
        const uintptr_t need = ar % 4 == 0 ? 16 : ar % 2 == 0 ? 8 : 4;
        if ((uintptr_t)mp % need)
            return fail(OP2G_ERR_INVALID, "map " + std::to_string(m) + " array is not " +
                                              std::to_string(need) + "-byte aligned");
    }
    return OP2G_OK;
}

op2g_status op2g_kernel_launch(op2g_kernel *k, const op2g_launch_desc *d, void *stream) {
    if (!k || !d) return fail(OP2G_ERR_INVALID, "NULL argument");
    if (d->end < d->start || d->start < 0) return fail(OP2G_ERR_INVALID, "bad iteration range");
    // parameter record: on the stack for the usual sizes (no heap
    // allocation per launch), on the heap for very long argument lists
    int64_t small[512];
    std::vector<int64_t> big;
    int64_t *buf = small;
    if ((size_t)k->param_bytes > sizeof small) {
        big.resize(k->param_bytes / 8);
        buf = big.data();
    }
    op2g_status st = op2g_kernel_pack_params(k, d, buf);
    if (st != OP2G_OK) return st;
    Loaded *L = nullptr;
    const bool al = use_aligned(k, d);
    st = load_module(al ? k->cubin_al : k->cubin, "op2g_wrap", "op2g_wrap_batched",
                     k->sig.block_size, al ? k->per_dev_al : k->per_dev, k->mu, &L);
    if (st != OP2G_OK) return st;
    if (k->staged) {
        if (d->end <= d->start) return OP2G_OK;
        // CTAs take mini-partitions in turn; the partitions' plan segments and
        // staged values take dynamic shared memory
        const size_t smem = staged_smem_bytes(k->sig, d->stage->block, d->stage->max_unique);
        Driver &D = driver();
        {
            std::lock_guard<std::mutex> g(k->mu);
            if ((int)smem > L->smem_attr && smem > 48 * 1024) {
                CUresult r = D.FuncSetAttribute(L->f, CU_FUNC_ATTRIBUTE_MAX_DYNAMIC_SHARED_SIZE_BYTES,
                                                (int)smem);
                if (r != CUDA_SUCCESS) return cu_fail(r, "cuFuncSetAttribute (shared memory)");
                L->smem_attr = (int)smem;
            }
            if (smem != L->occ_smem) {
                int occ = 0;
                if (D.OccupancyMaxActiveBlocksPerMultiprocessor(&occ, L->f, k->sig.block_size, smem) !=
                    CUDA_SUCCESS)
                    occ = 1;
                if (occ < 1)
                    return fail(OP2G_ERR_CAPACITY, "staged partitions need " + std::to_string(smem) +
                                                       " bytes of shared memory per CTA");
                L->occ_smem = smem;
                L->occ_at_smem = occ;
            }
        }
        const int64_t B = d->stage->block;
        const int64_t nparts = (d->end + B - 1) / B - d->start / B;
        // one resident wave: each CTA pipelines its partitions
        int64_t grid = d->grid > 0 ? d->grid
                       : d->grid < 0 ? nparts : (int64_t)L->occ_at_smem * L->sms;
        if (grid > nparts) grid = nparts;
        if (grid < 1) grid = 1;
        void *params[] = {buf};
        return launch(L->f, (unsigned)grid, (unsigned)k->sig.block_size, params, stream,
                      (unsigned)smem);
    }
    const int64_t per = d->layers_per_entity > 0 ? d->layers_per_entity : 1;
    const int64_t items = (d->end - d->start) * (k->sig.loop.extruded && k->sig.loop.constant_layers &&
                                                 column_parallel(k->sig) ? per : 1);
    if (items <= 0) return OP2G_OK;
    // a thread runs cells_per_thread iterations per sweep step: the grid is
    // sized for the steps
    const int64_t cpt = k->cells_per_thread > 1 ? k->cells_per_thread : 1;
    int32_t grid = 0, bs = 0, chunked = 0;
    op2g_launch_shape((items + cpt - 1) / cpt, (d->end - d->start + cpt - 1) / cpt,
                      k->sig.block_size, L->sms, L->occ, d->grid, L->fc != nullptr, &grid, &bs,
                      &chunked);
    void *params[] = {buf};
    return launch(chunked ? L->fc : L->f, (unsigned)grid, (unsigned)bs, params, stream);
}

void op2g_launch_shape(int64_t items, int64_t entities, int32_t block_size, int32_t sms,
                       int32_t ctas_per_sm, int32_t grid_request, int32_t chunked_available,
                       int32_t *grid_out, int32_t *block_out, int32_t *chunked_out) {
    int64_t bs = block_size > 0 ? block_size : 32;
    const int64_t nsm = sms > 0 ? sms : 1;
    if (entities < 1) entities = 1;
    if (items < 1) items = 1;
    // A launch of fewer than 4 full CTAs per SM runs the balanced entry: k
    // CTAs per SM (k = full CTAs per SM, rounded up), each taking an equal
    // contiguous chunk of the entities with as many threads as the chunk has
    // iterations (a multiple of 32, at most the compiled CTA size).  Small
    // loops then spread over every SM instead of a few full CTAs (each SM
    // issues FP64 at 2 per clock), and medium ones give every SM the same
    // work.  Wrappers with shared-memory staging have no balanced entry.
    const int64_t full = nsm * bs;
    if (grid_request == 0 && chunked_available && items < 4 * full) {
        int64_t g = nsm * ((items + full - 1) / full);
        if (g > entities) g = entities;
        const int64_t chunk = (entities + g - 1) / g;
        int64_t t = chunk * (items / entities);      // iterations per CTA
        t = (t + 31) / 32 * 32;
        if (t < bs) bs = t;
        *grid_out = (int32_t)g;
        *block_out = (int32_t)bs;
        *chunked_out = 1;
        return;
    }
    int64_t grid = grid_request > 0 ? grid_request : (items + bs - 1) / bs;
    // Default: up to 4 waves of resident CTAs.  Measured on GB300: one wave
    // leaves a tail of lone warps at the end of gather/scatter-bound loops
    // (10-14 % slower), while far more CTAs than that slow streaming loops.
    const int64_t cap = (int64_t)(ctas_per_sm > 0 ? ctas_per_sm : 1) * nsm * 4;
    if (grid_request == 0 && grid > cap) grid = cap;
    if (grid > INT32_MAX) grid = INT32_MAX;
    if (grid < 1) grid = 1;
    *grid_out = (int32_t)grid;
    *block_out = (int32_t)bs;
    *chunked_out = 0;
}

op2g_status op2g_kernel_launch_batched(op2g_kernel *k, const void *params_dev,
                                       const int64_t *work_dev, int64_t nwork, int32_t grid,
                                       void *stream) {
    if (!k || !params_dev || !work_dev) return fail(OP2G_ERR_INVALID, "NULL argument");
    if (nwork <= 0) return OP2G_OK;
    Loaded *L = nullptr;
    op2g_status st = load_module(k->cubin, "op2g_wrap", "op2g_wrap_batched", k->sig.block_size,
                                 k->per_dev, k->mu, &L);
    if (st != OP2G_OK) return st;
    int64_t g = grid > 0 ? grid : (int64_t)L->occ * L->sms;
    if (g > nwork) g = nwork;
    const void *p0 = params_dev;
    const int64_t *w0 = work_dev;
    long long nw = nwork;
    void *params[] = {(void *)&p0, (void *)&w0, (void *)&nw};
    return launch(L->fb, (unsigned)g, (unsigned)k->sig.block_size, params, stream);
}

}  // extern "C"

struct op2g_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" {

op2g_status op2g_graph_begin(void **capture_stream) {
    if (!capture_stream) return fail(OP2G_ERR_INVALID, "NULL argument");
    *capture_stream = nullptr;
    cudaStream_t s = nullptr;
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) return cuda_fail(e, "cudaStreamCreateWithFlags");
    // thread-local: other threads may keep using CUDA while this one records
    e = cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) {
        cudaStreamDestroy(s);
        return cuda_fail(e, "cudaStreamBeginCapture");
    }
    *capture_stream = (void *)s;
    return OP2G_OK;
}

op2g_status op2g_graph_end(void *capture_stream, op2g_graph **out) {
    if (!capture_stream) return fail(OP2G_ERR_INVALID, "NULL capture stream");
    if (out) *out = nullptr;
    cudaStream_t s = (cudaStream_t)capture_stream;
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &graph);
    cudaStreamDestroy(s);
    if (e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        return cuda_fail(e, "cudaStreamEndCapture");
    }
    if (!out) {
        cudaGraphDestroy(graph);
        return fail(OP2G_ERR_INVALID, "NULL output");
    }
    cudaGraphExec_t exec = nullptr;
    e = cudaGraphInstantiate(&exec, graph, 0);
    if (e != cudaSuccess) {
        cudaGraphDestroy(graph);
        return cuda_fail(e, "cudaGraphInstantiate");
    }
    op2g_graph *g = new op2g_graph;
    g->graph = graph;
    g->exec = exec;
    *out = g;
    return OP2G_OK;
}

op2g_status op2g_graph_launch(op2g_graph *g, void *stream) {
    if (!g || !g->exec) return fail(OP2G_ERR_INVALID, "NULL graph");
    cudaError_t e = cudaGraphLaunch(g->exec, (cudaStream_t)stream);
    if (e != cudaSuccess) return cuda_fail(e, "cudaGraphLaunch");
    return OP2G_OK;
}

void op2g_graph_destroy(op2g_graph *g) {
    if (!g) return;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
}

}  // extern "C"
