// op2g_device.cuh -- device-side building blocks of the generated par_loop
// wrappers.  This header is compiled by NVRTC together with the user's local
// kernel and the per-signature glue that op2g_codegen.cpp writes.  It holds the
// hand-written parts: typed pointers that convert to whatever pointer type the
// user's C kernel declares, the INC/MIN/MAX atomics for every element type,
// warp-level reductions for op2.Global arguments, warp-aggregated scatter and
// the block-CSR insertion used for op2.Mat arguments.
//
// Semantics follow the reference's sequential wrapper: pack, call, unpack
// (pyop2/codegen/builder.py:240-300 GlobalPack, :303-410 DatPack,
// :501-606 MatPack).
#pragma once

typedef signed char int8_t;
typedef unsigned char uint8_t;
typedef short int16_t;
typedef unsigned short uint16_t;
typedef int int32_t;
typedef unsigned int uint32_t;
typedef long long int64_t;
typedef unsigned long long uint64_t;

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif
#ifndef NULL
#define NULL 0
#endif

// C++ kernels (Kernel(..., cpp=True)) may call the <cmath> / <algorithm>
// names through std::.  NVRTC has no host standard headers (their #include
// lines are commented out by the wrapper generator), so the device math
// functions are made visible in namespace std here.
namespace std {
using ::abs; using ::fabs; using ::sqrt; using ::cbrt; using ::pow; using ::exp; using ::exp2;
using ::expm1; using ::log; using ::log2; using ::log10; using ::log1p; using ::sin; using ::cos;
using ::tan; using ::asin; using ::acos; using ::atan; using ::atan2; using ::sinh; using ::cosh;
using ::tanh; using ::floor; using ::ceil; using ::round; using ::trunc; using ::fmod;
using ::fmin; using ::fmax; using ::hypot; using ::erf; using ::erfc; using ::copysign;
using ::isnan; using ::isinf; using ::isfinite;
__device__ __forceinline__ double abs(double x) { return ::fabs(x); }
__device__ __forceinline__ float abs(float x) { return ::fabsf(x); }
template <class T> __device__ __forceinline__ const T &min(const T &a, const T &b) { return b < a ? b : a; }
template <class T> __device__ __forceinline__ const T &max(const T &a, const T &b) { return a < b ? b : a; }
}  // namespace std

namespace op2g {

// Kernel-argument pointer.  The reference passes every argument to the C
// kernel through a void*-typed ctypes call (pyop2/global_kernel.py:410-417),
// so a kernel may declare any pointer type for any argument; C++ would reject
// the implicit conversions, so the wrapper passes this proxy instead.
template <class T>
struct anyptr {
    T *p;
    __device__ __forceinline__ explicit anyptr(T *q) : p(q) {}
    template <class U>
    __device__ __forceinline__ operator U *() const { return (U *)p; }
};
template <class T>
__device__ __forceinline__ anyptr<T> ptr(T *p) { return anyptr<T>(p); }

__device__ __forceinline__ void set_err(int *err, int bit) {
    if (err) atomicOr(err, bit);
}

// ---------------------------------------------------------------- INC
__device__ __forceinline__ void atomic_inc(double *a, double v) { atomicAdd(a, v); }
__device__ __forceinline__ void atomic_inc(float *a, float v) { atomicAdd(a, v); }
__device__ __forceinline__ void atomic_inc(int *a, int v) { atomicAdd(a, v); }
__device__ __forceinline__ void atomic_inc(unsigned *a, unsigned v) { atomicAdd(a, v); }
__device__ __forceinline__ void atomic_inc(long long *a, long long v) {
    atomicAdd((unsigned long long *)a, (unsigned long long)v);
}
__device__ __forceinline__ void atomic_inc(unsigned long long *a, unsigned long long v) {
    atomicAdd(a, v);
}

// ------------------------------------------------------------ MIN/MAX
__device__ __forceinline__ void atomic_min(int *a, int v) { atomicMin(a, v); }
__device__ __forceinline__ void atomic_max(int *a, int v) { atomicMax(a, v); }
__device__ __forceinline__ void atomic_min(unsigned *a, unsigned v) { atomicMin(a, v); }
__device__ __forceinline__ void atomic_max(unsigned *a, unsigned v) { atomicMax(a, v); }
__device__ __forceinline__ void atomic_min(long long *a, long long v) { atomicMin(a, v); }
__device__ __forceinline__ void atomic_max(long long *a, long long v) { atomicMax(a, v); }
__device__ __forceinline__ void atomic_min(unsigned long long *a, unsigned long long v) {
    atomicMin(a, v);
}
__device__ __forceinline__ void atomic_max(unsigned long long *a, unsigned long long v) {
    atomicMax(a, v);
}
// Floating point MIN/MAX: compare-and-swap on the bit pattern.  The loop ends
// as soon as the stored value is already no larger (smaller) than v, so it
// performs at most one successful swap per distinct improvement.
__device__ __forceinline__ void atomic_min(double *a, double v) {
    unsigned long long *p = (unsigned long long *)a;
    unsigned long long old = *p;
    while (__longlong_as_double(old) > v) {
        unsigned long long seen = atomicCAS(p, old, __double_as_longlong(v));
        if (seen == old) break;
        old = seen;
    }
}
__device__ __forceinline__ void atomic_max(double *a, double v) {
    unsigned long long *p = (unsigned long long *)a;
    unsigned long long old = *p;
    while (__longlong_as_double(old) < v) {
        unsigned long long seen = atomicCAS(p, old, __double_as_longlong(v));
        if (seen == old) break;
        old = seen;
    }
}
__device__ __forceinline__ void atomic_min(float *a, float v) {
    int *p = (int *)a;
    int old = *p;
    while (__int_as_float(old) > v) {
        int seen = atomicCAS(p, old, __float_as_int(v));
        if (seen == old) break;
        old = seen;
    }
}
__device__ __forceinline__ void atomic_max(float *a, float v) {
    int *p = (int *)a;
    int old = *p;
    while (__int_as_float(old) < v) {
        int seen = atomicCAS(p, old, __float_as_int(v));
        if (seen == old) break;
        old = seen;
    }
}

template <class T>
__device__ __forceinline__ T vmin(T a, T b) { return b < a ? b : a; }
template <class T>
__device__ __forceinline__ T vmax(T a, T b) { return a < b ? b : a; }

// ------------------------------------------------- warp reductions (Globals)
template <class T>
__device__ __forceinline__ T shfl_xor(T v, int m) { return __shfl_xor_sync(0xffffffffu, v, m); }

template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v += shfl_xor(v, m);
    return v;
}
template <class T>
__device__ __forceinline__ T warp_min(T v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v = vmin(v, shfl_xor(v, m));
    return v;
}
template <class T>
__device__ __forceinline__ T warp_max(T v) {
#pragma unroll
    for (int m = 16; m > 0; m >>= 1) v = vmax(v, shfl_xor(v, m));
    return v;
}

// ------------------------------------------- warp-aggregated INC scatter
// All 32 lanes call this together (inactive lanes pass valid = false).  Lanes
// whose target address is equal form a group (__match_any_sync); the group's
// lowest lane sums the members' values in lane order with shuffles and issues
// one atomic.  The number of shuffle rounds is the size of the largest group.
template <class T>
__device__ __forceinline__ void warp_agg_inc(T *addr, T v, bool valid) {
    const unsigned lane = threadIdx.x & 31u;
    unsigned long long key = valid ? (unsigned long long)addr : 0ull;
    unsigned peers = __match_any_sync(0xffffffffu, key);
    const unsigned leader = __ffs(peers) - 1;
    const int gsize = __popc(peers);
    const int rounds = __reduce_max_sync(0xffffffffu, (unsigned)gsize);
    T acc = v;
    unsigned rest = peers & ~(1u << lane);   // members other than me
    for (int r = 1; r < rounds; ++r) {
        int src = rest ? (__ffs(rest) - 1) : (int)lane;
        T w = __shfl_sync(0xffffffffu, v, src);
        if (lane == leader && rest) acc += w;
        rest &= rest - 1u;
    }
    if (valid && lane == leader) atomic_inc(addr, acc);
}

// ------------------------------------------------------- block-CSR insertion
// Position of column `col` in block row `row` (binary search over the sorted
// unique column list), or -1 if absent.
__device__ __forceinline__ long long bcsr_find(const long long *__restrict__ rowptr,
                                               const int *__restrict__ colidx, int row, int col) {
    long long lo = rowptr[row], hi = rowptr[row + 1] - 1;
    while (lo <= hi) {
        long long mid = (lo + hi) >> 1;
        int c = colidx[mid];
        if (c == col) return mid;
        if (c < col) lo = mid + 1; else hi = mid - 1;
    }
    return -1;
}

// ------------------------------------------------- asynchronous staging copies
// Used by staged wrappers (OP2G_SCATTER_STAGED) to fetch the next
// partitions' data while the current one computes: bulk copies (the TMA's
// one-dimensional form) of contiguous plan segments completing on an
// mbarrier, and per-element asynchronous copies (cp.async) of gathered
// values, waited for by commit groups.
__device__ __forceinline__ unsigned smem_addr(const void *p) {
    return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}
// Order this thread's earlier generic-proxy accesses of shared memory before
// later asynchronous-proxy (bulk copy) accesses.
__device__ __forceinline__ void fence_proxy_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
                 "r"(bytes)
                 : "memory");
}
// dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes,
                                        unsigned long long *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}
// Wait for phase `parity` of the mbarrier to complete, giving up after a
// bounded number of tries (returns false then).
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity) {
    const unsigned a = smem_addr(bar);
    for (int it = 0; it < (1 << 20); ++it) {
        unsigned done;
        asm volatile(
            "{\n .reg .pred p_;\n mbarrier.try_wait.parity.shared::cta.b64 p_, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p_;\n}" : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}
template <int BYTES>
__device__ __forceinline__ void cp_async(void *dst, const void *src) {
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async moves 4, 8 or 16 bytes");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_addr(dst)), "l"(src),
                 "n"(BYTES)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

}  // namespace op2g
