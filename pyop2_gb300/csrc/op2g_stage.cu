// op2g_stage.cu -- the staging plan of a par_loop: mini-partitions of the
// iteration set with, per partition and map, the sorted list of distinct
// targets, and per map entry its slot in the partition's entries sorted by
// target.
//
// This is the "local renumbering and staging" part of the execution plan of
// the historical OP2 GPU backends (doc/sphinx/source/plan.rst:11-39; the
// generated CUDA stub that used it is shown in
// doc/sphinx/source/backends.rst:262-319): a partition's indirectly accessed
// data are staged once into shared memory through the distinct-target list
// (ind_map).  Where that backend coloured the threads of a partition to add
// INC contributions without conflicts, here every map entry owns one slot:
// the entries of a partition sorted by (target, position) are numbered
// 0 .. nvalid-1, the entries of one target form the run
// run_off[k] .. run_off[k + 1], and loc_map holds each entry's slot.  A
// kernel stores each contribution at its slot, then sums every run in slot
// order and adds the sum to the target once.  The plan is built on the GPU,
// one CTA per partition (a bitonic sort of (value, position) keys in shared
// memory).  Entries with negative values (PyOP2's "no target") get the slot
// 0xFFFF.  Each partition's segment of ind_map / run_off starts at a
// multiple of 8 entries (16-byte aligned), so segments can be bulk-copied.
#include <cuda_runtime.h>

#include <cstdint>
#include <string>

#include "op2g_internal.h"

namespace {

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return op2g::cuda_fail(e_, #call); \
    } while (0)

constexpr int PT = 512;           // threads of a plan CTA
constexpr int PMAX = 4096;        // map entries per partition (sorted in shared memory)
constexpr unsigned short NOLOC = 0xFFFF;

__device__ __forceinline__ unsigned long long key_of(int v, int pos) {
    return ((unsigned long long)(unsigned)v << 32) | (unsigned)pos;
}

// One CTA per partition.  pass 0: seg[b] = the partition's segment length
// (distinct count + 1, rounded up to 8) and num[b] = the distinct count;
// pass 1: the segment at ind_off[b] gets the distinct values (ind_map) and
// the first slot of each (run_off, plus the number of valid entries after
// the last), and loc_map[entry] = the entry's slot.
__global__ void __launch_bounds__(PT) k_stage_plan(long long n, int arity, const int *__restrict__ map,
                                                   long long block, int pass,
                                                   long long *__restrict__ seg,
                                                   int *__restrict__ num,
                                                   const long long *__restrict__ ind_off,
                                                   int *__restrict__ ind_map,
                                                   unsigned short *__restrict__ run_off,
                                                   unsigned short *__restrict__ loc_map) {
    __shared__ unsigned long long key[PMAX];
    __shared__ int tsum[PT];
    __shared__ int nvalid;
    const long long b = blockIdx.x;
    const long long c0 = b * block;
    const long long c1 = c0 + block < n ? c0 + block : n;
    const int ne = (int)((c1 - c0) * arity);          // <= PMAX (checked on the host)
    int np = 1;
    while (np < ne) np <<= 1;
    const int *src = map + c0 * arity;
    if (threadIdx.x == 0) nvalid = 0;
    __syncthreads();
    int myvalid = 0;
    for (int i = threadIdx.x; i < np; i += PT) {
        unsigned long long k = ~0ull;
        if (i < ne) {
            const int v = src[i];
            if (v >= 0) {
                k = key_of(v, i);
                ++myvalid;
            } else if (pass == 1) {
                loc_map[c0 * arity + i] = NOLOC;
            }
        }
        key[i] = k;
    }
    atomicAdd(&nvalid, myvalid);
    __syncthreads();
    // bitonic sort of np keys, ascending (invalid keys last)
    for (int size = 2; size <= np; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            for (int t = threadIdx.x; t < np / 2; t += PT) {
                const int lo = 2 * t - (t & (stride - 1));
                const int hi = lo + stride;
                const bool up = (lo & size) == 0;
                const unsigned long long a = key[lo], c = key[hi];
                if ((a > c) == up) {
                    key[lo] = c;
                    key[hi] = a;
                }
            }
            __syncthreads();
        }
    }
    // flags of first occurrences; each thread owns a contiguous run of keys
    const int per = (np + PT - 1) / PT;
    const int k0 = threadIdx.x * per;
    int mine = 0;
    for (int k = k0; k < k0 + per && k < np; ++k) {
        const unsigned long long x = key[k];
        if (x != ~0ull && (k == 0 || (key[k - 1] >> 32) != (x >> 32))) ++mine;
    }
    tsum[threadIdx.x] = mine;
    __syncthreads();
    // inclusive scan of the per-thread counts (Hillis-Steele)
    for (int o = 1; o < PT; o <<= 1) {
        const int y = threadIdx.x >= o ? tsum[threadIdx.x - o] : 0;
        __syncthreads();
        tsum[threadIdx.x] += y;
        __syncthreads();
    }
    const int nu = tsum[PT - 1];
    if (pass == 0) {
        if (threadIdx.x == 0) {
            seg[b] = (nu + 1 + 7) / 8 * 8;
            num[b] = nu;
        }
        return;
    }
    int local = (threadIdx.x ? tsum[threadIdx.x - 1] : 0) - 1;
    int *out = ind_map + ind_off[b];
    unsigned short *ro = run_off + ind_off[b];
    for (int k = k0; k < k0 + per && k < np; ++k) {
        const unsigned long long x = key[k];
        if (x == ~0ull) continue;
        if (k == 0 || (key[k - 1] >> 32) != (x >> 32)) {
            ++local;
            out[local] = (int)(x >> 32);
            ro[local] = (unsigned short)k;
        }
        loc_map[c0 * arity + (int)(x & 0xffffffffu)] = (unsigned short)k;
    }
    if (threadIdx.x == 0) ro[nu] = (unsigned short)nvalid;
}

__global__ void k_max_count(const int *__restrict__ c, long long n, unsigned *__restrict__ mx) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    unsigned m = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += stride)
        m = (unsigned)c[i] > m ? (unsigned)c[i] : m;
    atomicMax(mx, m);
}

size_t a256(size_t x) { return (x + 255) & ~(size_t)255; }

op2g_status check_args(int64_t n, int32_t arity, int64_t block) {
    if (n < 0 || arity <= 0 || block <= 0)
        return op2g::fail(OP2G_ERR_INVALID, "staging plan: bad sizes");
    if (block * arity > PMAX)
        return op2g::fail(OP2G_ERR_INVALID, "staging plan: block x arity above " +
                                                std::to_string(PMAX));
    return OP2G_OK;
}

}  // namespace

extern "C" {

op2g_status op2g_stage_plan_workspace(int64_t n, int32_t arity, int64_t block, size_t *bytes) {
    op2g_status s = check_args(n, arity, block);
    if (s != OP2G_OK) return s;
    const long long nb = (n + block - 1) / block;
    size_t off = a256(sizeof(long long) * op2g::scan_tmp_elems(nb + 1));  // scan temp
    off = a256(off + 64);                                                  // max
    if (bytes) *bytes = off;
    return OP2G_OK;
}

op2g_status op2g_stage_plan_count(int64_t n, int32_t arity, const int32_t *map, int64_t block,
                                  void *ws, size_t ws_bytes, int64_t *ind_off, int32_t *ind_num,
                                  int64_t *total, int32_t *max_unique, void *stream) {
    op2g_status s = check_args(n, arity, block);
    if (s != OP2G_OK) return s;
    size_t need = 0;
    op2g_stage_plan_workspace(n, arity, block, &need);
    if (!ws || ws_bytes < need) return op2g::fail(OP2G_ERR_INVALID, "workspace too small");
    const long long nb = (n + block - 1) / block;
    if (!ind_off || (nb > 0 && (!map || !ind_num)))
        return op2g::fail(OP2G_ERR_INVALID, "NULL argument");
    cudaStream_t st = (cudaStream_t)stream;
    long long *tmp = (long long *)ws;
    unsigned *mx =
        (unsigned *)((char *)ws + a256(sizeof(long long) * op2g::scan_tmp_elems(nb + 1)));
    CK(cudaMemsetAsync(ind_off, 0, sizeof(long long) * (nb + 1), st));
    CK(cudaMemsetAsync(mx, 0, sizeof(unsigned), st));
    if (nb > 0) {
        k_stage_plan<<<(unsigned)nb, PT, 0, st>>>(n, arity, map, block, 0, (long long *)ind_off,
                                                  ind_num, nullptr, nullptr, nullptr, nullptr);
        CK(cudaGetLastError());
        k_max_count<<<nb < 1024 ? 1 : 152, 256, 0, st>>>(ind_num, nb, mx);
        CK(cudaGetLastError());
    }
    s = op2g::scan_exclusive((long long *)ind_off, nb + 1, tmp, st);
    if (s != OP2G_OK) return s;
    long long tot = 0;
    unsigned m = 0;
    CK(cudaMemcpyAsync(&tot, ind_off + nb, sizeof tot, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&m, mx, sizeof m, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (total) *total = tot;
    if (max_unique) *max_unique = (int32_t)m;
    return OP2G_OK;
}

op2g_status op2g_stage_plan_fill(int64_t n, int32_t arity, const int32_t *map, int64_t block,
                                 const int64_t *ind_off, int32_t *ind_map, uint16_t *run_off,
                                 uint16_t *loc_map, void *stream) {
    op2g_status s = check_args(n, arity, block);
    if (s != OP2G_OK) return s;
    if (n == 0) return OP2G_OK;
    if (!map || !ind_off || !ind_map || !run_off || !loc_map)
        return op2g::fail(OP2G_ERR_INVALID, "NULL argument");
    cudaStream_t st = (cudaStream_t)stream;
    const long long nb = (n + block - 1) / block;
    k_stage_plan<<<(unsigned)nb, PT, 0, st>>>(n, arity, map, block, 1, nullptr, nullptr,
                                              (const long long *)ind_off, ind_map, run_off,
                                              loc_map);
    CK(cudaGetLastError());
    return OP2G_OK;
}

}  // extern "C"
