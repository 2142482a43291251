// op2g_kernels.cu -- hand-written sm_103a kernels behind the non-par_loop parts
// of the C ABI: the Map -> block-CSR sparsity build, block-CSR matrix
// utilities, greedy colouring, a prefix scan shared by them, and the FP64
// throughput probe used as the second roofline ceiling.
//
// Sparsity semantics restate pyop2/sparsity.pyx:178-405 (fill_with_zeros):
// every (row map, column map, iteration region) triple inserts the block
// rmap[e,:] x cmap[e,:] for every iterated entity (and layer), composed maps
// are resolved innermost-last and skipped when negative (:249-259, :270-281),
// extruded maps add offset * ((layer + k + q) % nl - q % nl) (:361-374), the
// diagonal (i, i) is added for i < min(nrows, ncols) when requested
// (:214-219), and negative indices are ignored as PETSc's MatSetValues does.
// The result is PETSc's preallocated pattern: per row, the sorted set of
// distinct columns.
#include <cuda_runtime.h>

#include <climits>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "op2g_internal.h"

namespace {

constexpr int MAXAR = 128;  // arity bound for extruded offset tables

struct PairDev {
    const int *rmap, *cmap;
    int rarity, carity;
    long long nent;
    int region;
    int nrc, ncc;
    const int *rc[OP2G_MAX_COMPOSED];
    const int *cc[OP2G_MAX_COMPOSED];
    int has_roff, has_coff;
    int tr, tc;          // rows / columns of one virtual cell (x2 for interior facets)
    long long nvirt;     // virtual cells (entities x layer slots)
    int roff[MAXAR], coff[MAXAR], rq[MAXAR], cq[MAXAR];
};

struct SpDev {
    long long nrows, ncols;
    int set_diag, extruded, constant_layers, periodic;
    const int *layers;
    int slots;
    int *err;
};

#define CK(call)                                                   \
    do {                                                           \
        cudaError_t e_ = (call);                                   \
        if (e_ != cudaSuccess) return op2g::cuda_fail(e_, #call); \
    } while (0)

__device__ __forceinline__ bool vcell(const SpDev &S, const PairDev &P, long long v,
                                      long long &rent, long long &cent, int &layer, int &nl) {
    const long long e = S.extruded ? v / S.slots : v;
    const int l = S.extruded ? (int)(v - e * S.slots) : 0;
    rent = e;
    cent = e;
    for (int i = 0; i < P.nrc; ++i) {
        rent = P.rc[P.nrc - 1 - i][rent];
        if (rent < 0) return false;
    }
    for (int i = 0; i < P.ncc; ++i) {
        cent = P.cc[P.ncc - 1 - i][cent];
        if (cent < 0) return false;
    }
    layer = 0;
    nl = 1;
    if (S.extruded) {
        const int *L = S.constant_layers ? S.layers : S.layers + 2 * e;
        int ls = L[0], le = L[1] - 1;
        nl = le - ls;
        if (P.region == OP2G_ON_BOTTOM) le = ls + 1;
        else if (P.region == OP2G_ON_TOP) ls = le - 1;
        else if (P.region == OP2G_ON_INTERIOR_FACETS && !S.periodic) le = le - 1;
        layer = ls + l;
        if (layer >= le) return false;
    }
    return true;
}

__device__ __forceinline__ int ext_term(int layer, int k, int q, int nl) {
    const int eff = layer + k + q;
    return nl > 0 ? (eff % nl - q % nl) : (eff - q);
}

// Row (column) of local entry ir (jr) of facet k of a virtual cell: the
// map value plus the extruded offset term.
__device__ __forceinline__ int row_of(const SpDev &S, const PairDev &P, long long rent, int k,
                                      int ir, int layer, int nl) {
    int b = __ldg(P.rmap + rent * P.rarity + ir);
    if (S.extruded && P.has_roff) b += P.roff[ir] * ext_term(layer, k, P.rq[ir], nl);
    return b;
}

__device__ __forceinline__ int col_of(const SpDev &S, const PairDev &P, long long cent, int k,
                                      int jr, int layer, int nl) {
    int b = __ldg(P.cmap + cent * P.carity + jr);
    if (S.extruded && P.has_coff) b += P.coff[jr] * ext_term(layer, k, P.cq[jr], nl);
    return b;
}

// Row -> virtual-cell incidence: counts (pass 0) or fills (pass 1).
// With a single pair every incidence brings the same number of candidate
// columns (tc), so the candidate counts follow from the incidence counts
// and cand is left untouched (one atomic per incidence instead of two).
// narrow: the transpose list holds 32-bit entity numbers (one pair over a
// flat set), otherwise 64-bit codes (pair << 56 | virtual cell).
__global__ void k_incidence(SpDev S, const PairDev *__restrict__ pairs, int p, int pass,
                            int single_pair, int narrow, long long *__restrict__ cnt,
                            int *__restrict__ cand, int *__restrict__ fillpos,
                            long long *__restrict__ tlist) {
    const PairDev &P = pairs[p];
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < P.nvirt; v += stride) {
        long long rent, cent;
        int layer, nl;
        if (!vcell(S, P, v, rent, cent, layer, nl)) continue;
        const int ra = P.rarity, nfr = P.tr / ra;
        for (int i = 0; i < P.tr; ++i) {
            const int k = nfr == 1 ? 0 : (i >= ra);
            const int r = row_of(S, P, rent, k, i - k * ra, layer, nl);
            if (r < 0) continue;
            if (r >= S.nrows) {
                atomicOr(S.err, OP2G_DEVERR_MAP_BOUNDS);
                continue;
            }
            if (pass == 0) {
                atomicAdd((unsigned long long *)&cnt[r], 1ull);
                if (!single_pair) atomicAdd(&cand[r], P.tc);
            } else {
                const long long pos = cnt[r] + atomicAdd(&fillpos[r], 1);
                if (narrow)
                    ((int *)tlist)[pos] = (int)v;
                else
                    tlist[pos] = ((long long)p << 56) | v;
            }
        }
    }
}

// Candidate count of row i: cand[i], or its incidences times tc when tc > 0
// (one pair); cnt holds the scanned incidence offsets by then.
__device__ __forceinline__ long long cand_of(const int *cand, const long long *cnt, int tc,
                                             long long i) {
    return tc > 0 ? (cnt[i + 1] - cnt[i]) * tc : (long long)cand[i];
}

__global__ void k_max_cand(const int *__restrict__ cand, const long long *__restrict__ cnt,
                           int tc, long long n, int diag, int *out) {
    int m = 0;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        m = max(m, (int)cand_of(cand, cnt, tc, i) + diag);
    for (int o = 16; o > 0; o >>= 1) m = max(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0) atomicMax(out, m);
}

// One warp per row: insert the candidate columns of every incident virtual
// cell into a per-warp open-addressing hash table in shared memory (empty
// slot = -1, linear probing, table at least twice the largest candidate
// count), collecting each first occurrence into a list; sort the distinct
// columns (rank sort with shuffles when they fit a warp, bitonic otherwise)
// and store them at the row's candidate offset.  A mesh row has ~100
// candidates but ~15 distinct columns, so only the distinct ones are sorted.
constexpr int ROW_HDR = 32;  // per-warp header ints (distinct counter)

__device__ __forceinline__ unsigned col_hash(int c, unsigned mask) {
    return ((unsigned)c * 2654435761u) & mask;
}

__device__ __forceinline__ void row_insert(int c, int *tab, unsigned mask, int tsize, int *uniq,
                                           int *uslot, int *ucount, int *err) {
    unsigned h = col_hash(c, mask);
    for (int probe = 0; probe < tsize; ++probe) {
        const int old = atomicCAS(&tab[h], -1, c);
        if (old == -1) {
            const int k = atomicAdd(ucount, 1);
            uniq[k] = c;
            uslot[k] = (int)h;
            return;
        }
        if (old == c) return;
        h = (h + 1) & mask;
    }
    atomicOr(err, OP2G_DEVERR_CAPACITY);  // table full: cannot happen (tsize >= 2 x candidates)
}

// SIMPLE: one (row map, column map) pair over a flat set with no composed
// maps, so the transpose list holds 32-bit entity numbers and an entry's
// candidate columns are one row of the column map.  The warp then walks the incident
// cells in warp-uniform rounds and, per column slot, lets only the first of
// the lanes holding the same column insert it (__match_any_sync): on a mesh
// a vertex's own column recurs in every incident cell, and most neighbours
// in several, so this removes about half of the shared-memory atomics.
template <bool SIMPLE>
__global__ void k_rows(SpDev S, const PairDev *__restrict__ pairs,
                       const long long *__restrict__ tptr, const long long *__restrict__ tlist,
                       int tsize, int ucap, const long long *__restrict__ candptr,
                       int *__restrict__ tmp, long long *__restrict__ rowcount) {
    extern __shared__ int smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int wpb = blockDim.x >> 5;
    int *hdr = smem + warp * (ROW_HDR + tsize + 2 * ucap);
    int *tab = hdr + ROW_HDR;
    int *uniq = tab + tsize;
    int *uslot = uniq + ucap;     // table slot claimed by each distinct column
    const unsigned mask = (unsigned)tsize - 1u;
    // the table is emptied once here and afterwards only at the slots a row
    // claimed (~15 of tsize)
    for (int i = lane; i < tsize; i += 32) tab[i] = -1;
    for (long long r = (long long)blockIdx.x * wpb + warp; r < S.nrows;
         r += (long long)gridDim.x * wpb) {
        if (lane == 0) hdr[0] = 0;
        __syncwarp();
        const long long e0 = tptr[r], e1 = tptr[r + 1];
        if (SIMPLE) {
            const int *cmap = pairs[0].cmap;
            const int ca = pairs[0].carity;
            for (long long b = e0; b < e1; b += 32) {  // warp-uniform rounds
                const long long e = b + lane;
                const int *crow =
                    e < e1 ? cmap + (long long)((const int *)tlist)[e] * ca : nullptr;
                for (int j = 0; j < ca; ++j) {
                    int c = crow ? __ldg(crow + j) : -1;
                    if (c >= S.ncols) {
                        atomicOr(S.err, OP2G_DEVERR_MAP_BOUNDS);
                        c = -1;
                    }
                    const unsigned same = __match_any_sync(0xffffffffu, c);
                    if (c >= 0 && (__ffs(same) - 1) == lane)
                        row_insert(c, tab, mask, tsize, uniq, uslot, hdr, S.err);
                }
            }
        }
        for (long long e = e0 + lane; !SIMPLE && e < e1; e += 32) {
            const long long code = tlist[e];
            const PairDev &P = pairs[(int)(code >> 56)];
            long long rent, cent;
            int layer, nl;
            if (!vcell(S, P, code & ((1ll << 56) - 1), rent, cent, layer, nl)) continue;
            const int ca = P.carity, nfc = P.tc / ca;
            for (int j = 0; j < P.tc; ++j) {
                const int k = nfc == 1 ? 0 : (j >= ca);
                const int c = col_of(S, P, cent, k, j - k * ca, layer, nl);
                if (c < 0) continue;
                if (c >= S.ncols) {
                    atomicOr(S.err, OP2G_DEVERR_MAP_BOUNDS);
                    continue;
                }
                row_insert(c, tab, mask, tsize, uniq, uslot, hdr, S.err);
            }
        }
        if (S.set_diag && r < S.ncols && lane == 0)
            row_insert((int)r, tab, mask, tsize, uniq, uslot, hdr, S.err);
        __syncwarp();
        const int u = hdr[0];
        int *out = tmp + candptr[r];
        if (u <= 32) {
            // rank sort over the u distinct columns (u is warp-uniform)
            const int x = lane < u ? uniq[lane] : INT_MAX;
            int rank = 0;
            for (int j = 0; j < u; ++j) rank += __shfl_sync(0xffffffffu, x, j) < x;
            if (lane < u) out[rank] = x;
        } else {
            int P2 = 1;
            while (P2 < u) P2 <<= 1;
            for (int i = u + lane; i < P2; i += 32) uniq[i] = INT_MAX;
            __syncwarp();
            for (int k = 2; k <= P2; k <<= 1)
                for (int j = k >> 1; j > 0; j >>= 1) {
                    for (int i = lane; i < P2; i += 32) {
                        const int ixj = i ^ j;
                        if (ixj > i) {
                            const int a = uniq[i], b = uniq[ixj];
                            if ((a > b) == ((i & k) == 0)) {
                                uniq[i] = b;
                                uniq[ixj] = a;
                            }
                        }
                    }
                    __syncwarp();
                }
            for (int i = lane; i < u; i += 32) out[i] = uniq[i];
        }
        if (lane == 0) rowcount[r] = u;
        for (int i = lane; i < u; i += 32) tab[uslot[i]] = -1;
        __syncwarp();
    }
}

// candptr[r] = cand[r] + (diagonal entry of row r), to be scanned.
__global__ void k_cand_sizes(const int *__restrict__ cand, const long long *__restrict__ cnt,
                             int tc, long long n, long long ncols, int diag,
                             long long *__restrict__ candptr) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < n; r += stride)
        candptr[r] = cand_of(cand, cnt, tc, r) + ((diag && r < ncols) ? 1 : 0);
}

// One warp per row: copy the sorted distinct columns to the CSR column array.
__global__ void k_rows_copy(long long nrows, const long long *__restrict__ candptr,
                            const int *__restrict__ tmp, const long long *__restrict__ rowptr,
                            int *__restrict__ colidx) {
    const int lane = threadIdx.x & 31;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long r = w0; r < nrows; r += nw) {
        const long long o = rowptr[r], n = rowptr[r + 1] - o, c0 = candptr[r];
        for (long long i = lane; i < n; i += 32) colidx[o + i] = tmp[c0 + i];
    }
}

}  // namespace

namespace op2g {

// ---------------------------------------------------------------- scan
// (shared with the staging plan in op2g_stage.cu)
constexpr int SCAN_T = 1024, SCAN_V = 4, SCAN_B = SCAN_T * SCAN_V;

__global__ void __launch_bounds__(SCAN_T) k_scan_block(long long *__restrict__ d, long long n,
                                                       long long *__restrict__ sums) {
    __shared__ long long ws[32];
    const long long b0 = (long long)blockIdx.x * SCAN_B + (long long)threadIdx.x * SCAN_V;
    long long v[SCAN_V], t = 0;
#pragma unroll
    for (int k = 0; k < SCAN_V; ++k) {
        v[k] = (b0 + k < n) ? d[b0 + k] : 0;
        t += v[k];
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    long long inc = t;
    for (int o = 1; o < 32; o <<= 1) {
        long long y = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += y;
    }
    if (lane == 31) ws[w] = inc;
    __syncthreads();
    if (w == 0) {
        long long x = ws[lane];
        for (int o = 1; o < 32; o <<= 1) {
            long long y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        ws[lane] = x;
    }
    __syncthreads();
    long long run = inc - t + (w ? ws[w - 1] : 0);
#pragma unroll
    for (int k = 0; k < SCAN_V; ++k) {
        if (b0 + k < n) d[b0 + k] = run;
        run += v[k];
    }
    if (sums && threadIdx.x == SCAN_T - 1) sums[blockIdx.x] = run;
}

__global__ void k_scan_add(long long *__restrict__ d, long long n, const long long *__restrict__ offs) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) d[i] += offs[i / SCAN_B];
}

size_t scan_tmp_elems(long long n) {
    size_t tot = 0;
    while (n > SCAN_B) {
        n = (n + SCAN_B - 1) / SCAN_B;
        tot += (size_t)n;
    }
    return tot + 1;
}

// Exclusive in-place scan of d[0..n); tmp needs scan_tmp_elems(n) elements.
op2g_status scan_exclusive(long long *d, long long n, long long *tmp, cudaStream_t st) {
    if (n <= 0) return OP2G_OK;
    if (n <= SCAN_B) {
        k_scan_block<<<1, SCAN_T, 0, st>>>(d, n, nullptr);
        CK(cudaGetLastError());
        return OP2G_OK;
    }
    const long long nb = (n + SCAN_B - 1) / SCAN_B;
    k_scan_block<<<(unsigned)nb, SCAN_T, 0, st>>>(d, n, tmp);
    CK(cudaGetLastError());
    op2g_status s = scan_exclusive(tmp, nb, tmp + nb, st);
    if (s != OP2G_OK) return s;
    k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(d, n, tmp);
    CK(cudaGetLastError());
    return OP2G_OK;
}

}  // namespace op2g

namespace {

using op2g::scan_exclusive;
using op2g::scan_tmp_elems;

// ------------------------------------------------------- sparsity driver
struct SpLayout {
    size_t off_cnt, off_cand, off_fill, off_tlist, off_scan, off_pairs, off_misc, off_candptr,
        off_tmp, total;
    long long ninc, ncand;
};

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

op2g_status sp_prepare(const op2g_sparsity_desc *d, std::vector<PairDev> &pairs, SpDev &S,
                       SpLayout &L) {
    if (!d || d->npairs < 0 || (d->npairs && !d->pairs))
        return op2g::fail(OP2G_ERR_INVALID, "bad sparsity descriptor");
    if (d->nrows < 0 || d->ncols < 0 || d->nrows > INT_MAX || d->ncols > INT_MAX)
        return op2g::fail(OP2G_ERR_INVALID, "row/column counts must fit int32");
    if (d->npairs > 255) return op2g::fail(OP2G_ERR_INVALID, "at most 255 map pairs");
    memset(&S, 0, sizeof S);
    S.nrows = d->nrows;
    S.ncols = d->ncols;
    S.set_diag = d->set_diag;
    S.extruded = d->extruded;
    S.constant_layers = d->constant_layers;
    S.periodic = d->extruded_periodic;
    S.layers = d->layers;
    S.slots = d->extruded ? (d->layer_slots > 0 ? d->layer_slots : 1) : 1;
    if (d->extruded && !d->layers) return op2g::fail(OP2G_ERR_INVALID, "extruded sparsity needs layers");
    L.ninc = 0;
    L.ncand = 0;
    pairs.resize(d->npairs);
    for (int p = 0; p < d->npairs; ++p) {
        const op2g_sparsity_pair &q = d->pairs[p];
        PairDev &P = pairs[p];
        memset(&P, 0, sizeof P);
        if (!q.rmap || !q.cmap || q.rarity <= 0 || q.carity <= 0 || q.nent < 0)
            return op2g::fail(OP2G_ERR_INVALID, "bad map pair");
        if (q.nrcomposed < 0 || q.nrcomposed > OP2G_MAX_COMPOSED || q.nccomposed < 0 ||
            q.nccomposed > OP2G_MAX_COMPOSED)
            return op2g::fail(OP2G_ERR_INVALID, "bad composed chain");
        P.rmap = q.rmap;
        P.cmap = q.cmap;
        P.rarity = q.rarity;
        P.carity = q.carity;
        P.nent = q.nent;
        P.region = q.region ? q.region : OP2G_ALL;
        P.nrc = q.nrcomposed;
        P.ncc = q.nccomposed;
        for (int k = 0; k < OP2G_MAX_COMPOSED; ++k) {
            P.rc[k] = q.rcomposed[k];
            P.cc[k] = q.ccomposed[k];
        }
        const int ih = (d->extruded && P.region == OP2G_ON_INTERIOR_FACETS) ? 2 : 1;
        P.tr = ih * q.rarity;
        P.tc = ih * q.carity;
        if (d->extruded) {
            if (q.rarity > MAXAR || q.carity > MAXAR)
                return op2g::fail(OP2G_ERR_UNSUPPORTED, "extruded sparsity supports arity <= 128");
            if (!q.roffset || !q.coffset)
                return op2g::fail(OP2G_ERR_INVALID, "extruded sparsity needs map offsets");
            P.has_roff = P.has_coff = 1;
            for (int i = 0; i < q.rarity; ++i) {
                P.roff[i] = q.roffset[i];
                P.rq[i] = q.roffset_quotient ? q.roffset_quotient[i] : 0;
            }
            for (int i = 0; i < q.carity; ++i) {
                P.coff[i] = q.coffset[i];
                P.cq[i] = q.coffset_quotient ? q.coffset_quotient[i] : 0;
            }
        }
        P.nvirt = q.nent * S.slots;
        L.ninc += P.nvirt * P.tr;
        L.ncand += P.nvirt * P.tr * P.tc;
    }
    L.ncand += d->nrows;  // diagonal entries
    const long long n1 = d->nrows + 1;
    size_t off = 0;
    L.off_cnt = off; off = align256(off + sizeof(long long) * n1);
    L.off_cand = off; off = align256(off + sizeof(int) * (d->nrows + 1));
    L.off_fill = off; off = align256(off + sizeof(int) * (d->nrows + 1));
    L.off_tlist = off; off = align256(off + sizeof(long long) * (L.ninc > 0 ? L.ninc : 1));
    L.off_scan = off; off = align256(off + sizeof(long long) * scan_tmp_elems(n1));
    L.off_pairs = off; off = align256(off + sizeof(PairDev) * (d->npairs ? d->npairs : 1));
    L.off_misc = off; off = align256(off + 64);
    L.off_candptr = off; off = align256(off + sizeof(long long) * n1);
    L.off_tmp = off; off = align256(off + sizeof(int) * (L.ncand > 0 ? L.ncand : 1));
    L.total = off;
    return OP2G_OK;
}

int sms_of_current() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 1;
}

op2g_status sp_rows_launch(const SpDev &S, const PairDev *pd, bool simple,
                           const long long *tptr, const long long *tlist, int max_cand,
                           const long long *candptr, int *tmp, long long *rowcount,
                           cudaStream_t st) {
    if (S.nrows == 0) return OP2G_OK;
    int tsize = 32;
    while (tsize < 2 * max_cand) tsize <<= 1;
    int ucap = 32;
    while (ucap < max_cand) ucap <<= 1;
    const size_t per = (size_t)(ROW_HDR + tsize + 2 * ucap) * sizeof(int);
    int wpb = (int)((48 * 1024) / per);
    if (wpb > 8) wpb = 8;
    if (wpb < 1) wpb = 1;
    const size_t smem = per * wpb;
    if (smem > 227 * 1024)
        return op2g::fail(OP2G_ERR_CAPACITY, "a sparsity row has more than 18,000 candidate columns");
    if (smem > 48 * 1024) {
        CK(cudaFuncSetAttribute(k_rows<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
        CK(cudaFuncSetAttribute(k_rows<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)smem));
    }
    long long blocks = (S.nrows + wpb - 1) / wpb;
    const long long capb = (long long)sms_of_current() * 32;
    if (blocks > capb) blocks = capb;
    if (simple)
        k_rows<true><<<(unsigned)blocks, 32 * wpb, smem, st>>>(S, pd, tptr, tlist, tsize, ucap,
                                                               candptr, tmp, rowcount);
    else
        k_rows<false><<<(unsigned)blocks, 32 * wpb, smem, st>>>(S, pd, tptr, tlist, tsize, ucap,
                                                                candptr, tmp, rowcount);
    CK(cudaGetLastError());
    return OP2G_OK;
}

unsigned grid_for_rows(long long nrows) {
    long long g = (nrows * 32 + 255) / 256;
    const long long cap = (long long)sms_of_current() * 16;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

// State kept in the workspace between count and fill (the candidate capacity).
struct SpMisc {
    int max_cand;
    int err;
    int cap;
};

}  // namespace

extern "C" {

op2g_status op2g_sparsity_workspace(const op2g_sparsity_desc *d, size_t *bytes) {
    std::vector<PairDev> pairs;
    SpDev S;
    SpLayout L;
    op2g_status s = sp_prepare(d, pairs, S, L);
    if (s != OP2G_OK) return s;
    if (bytes) *bytes = L.total;
    return OP2G_OK;
}

op2g_status op2g_sparsity_count(const op2g_sparsity_desc *d, void *ws, size_t ws_bytes,
                                int64_t *rowptr, int64_t *nnz, void *stream) {
    std::vector<PairDev> pairs;
    SpDev S;
    SpLayout L;
    op2g_status s = sp_prepare(d, pairs, S, L);
    if (s != OP2G_OK) return s;
    if (!ws || ws_bytes < L.total) return op2g::fail(OP2G_ERR_INVALID, "workspace too small");
    if (!rowptr) return op2g::fail(OP2G_ERR_INVALID, "rowptr is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    char *w = (char *)ws;
    long long *cnt = (long long *)(w + L.off_cnt);
    int *cand = (int *)(w + L.off_cand);
    int *fill = (int *)(w + L.off_fill);
    long long *tlist = (long long *)(w + L.off_tlist);
    long long *scan = (long long *)(w + L.off_scan);
    PairDev *pd = (PairDev *)(w + L.off_pairs);
    SpMisc *misc = (SpMisc *)(w + L.off_misc);
    S.err = &misc->err;
    const long long n1 = d->nrows + 1;
    CK(cudaMemsetAsync(cnt, 0, sizeof(long long) * n1, st));
    CK(cudaMemsetAsync(cand, 0, sizeof(int) * n1, st));
    CK(cudaMemsetAsync(fill, 0, sizeof(int) * n1, st));
    CK(cudaMemsetAsync(misc, 0, sizeof(SpMisc), st));
    if (!pairs.empty())
        CK(cudaMemcpyAsync(pd, pairs.data(), sizeof(PairDev) * pairs.size(), cudaMemcpyHostToDevice, st));
    const long long capb = (long long)sms_of_current() * 16;
    const int single = pairs.size() == 1 ? 1 : 0;
    const int tc1 = single ? pairs[0].tc : 0;  // candidates per incidence with one pair
    // one pair over a flat set without composed maps: the transpose list
    // holds entity numbers (32-bit: set sizes are int32)
    const bool simple = single && !d->extruded && pairs[0].nrc == 0 && pairs[0].ncc == 0;
    for (int pass = 0; pass < 2; ++pass) {
        for (size_t p = 0; p < pairs.size(); ++p) {
            long long nb = (pairs[p].nvirt + 255) / 256;
            if (nb == 0) continue;
            if (nb > capb) nb = capb;
            k_incidence<<<(unsigned)nb, 256, 0, st>>>(S, pd, (int)p, pass, single,
                                                      simple ? 1 : 0, cnt, cand, fill, tlist);
            CK(cudaGetLastError());
        }
        if (pass == 0) {
            s = scan_exclusive(cnt, n1, scan, st);
            if (s != OP2G_OK) return s;
        }
    }
    if (d->nrows > 0) {
        long long nb = (d->nrows + 255) / 256;
        if (nb > capb) nb = capb;
        k_max_cand<<<(unsigned)nb, 256, 0, st>>>(cand, cnt, tc1, d->nrows, d->set_diag ? 1 : 0,
                                                 &misc->max_cand);
        CK(cudaGetLastError());
    }
    SpMisc hm;
    CK(cudaMemcpyAsync(&hm, misc, sizeof hm, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (hm.err & OP2G_DEVERR_MAP_BOUNDS)
        return op2g::fail(OP2G_ERR_BOUNDS, "a map value is outside the row or column set");
    // candidate offsets (upper bound of each row's distinct columns)
    long long *candptr = (long long *)(w + L.off_candptr);
    int *tmp = (int *)(w + L.off_tmp);
    {
        long long nb = (d->nrows + 255) / 256;
        if (nb > capb) nb = capb;
        if (nb < 1) nb = 1;
        k_cand_sizes<<<(unsigned)nb, 256, 0, st>>>(cand, cnt, tc1, d->nrows, d->ncols,
                                                   d->set_diag ? 1 : 0,
                                                   candptr);
        CK(cudaGetLastError());
        CK(cudaMemsetAsync(candptr + d->nrows, 0, sizeof(long long), st));
        s = scan_exclusive(candptr, n1, scan, st);
        if (s != OP2G_OK) return s;
    }
    int cap = hm.max_cand > 1 ? hm.max_cand : 1;
    CK(cudaMemcpyAsync(&misc->cap, &cap, sizeof(int), cudaMemcpyHostToDevice, st));
    s = sp_rows_launch(S, pd, simple, cnt, tlist, cap, candptr, tmp, (long long *)rowptr, st);
    if (s != OP2G_OK) return s;
    CK(cudaMemsetAsync(rowptr + d->nrows, 0, sizeof(long long), st));
    s = scan_exclusive((long long *)rowptr, n1, scan, st);
    if (s != OP2G_OK) return s;
    long long total = 0;
    int err = 0;
    CK(cudaMemcpyAsync(&total, rowptr + d->nrows, sizeof total, cudaMemcpyDeviceToHost, st));
    CK(cudaMemcpyAsync(&err, &misc->err, sizeof err, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (err & OP2G_DEVERR_MAP_BOUNDS)
        return op2g::fail(OP2G_ERR_BOUNDS, "a map value is outside the row or column set");
    if (err & OP2G_DEVERR_CAPACITY)
        return op2g::fail(OP2G_ERR_CAPACITY, "sparsity row candidate capacity exceeded");
    if (nnz) *nnz = total;
    return OP2G_OK;
}

op2g_status op2g_sparsity_fill(const op2g_sparsity_desc *d, void *ws, size_t ws_bytes,
                               const int64_t *rowptr, int32_t *colidx, void *stream) {
    std::vector<PairDev> pairs;
    SpDev S;
    SpLayout L;
    op2g_status s = sp_prepare(d, pairs, S, L);
    if (s != OP2G_OK) return s;
    if (!ws || ws_bytes < L.total) return op2g::fail(OP2G_ERR_INVALID, "workspace too small");
    if (!rowptr || (!colidx && d->nrows > 0)) return op2g::fail(OP2G_ERR_INVALID, "NULL output");
    cudaStream_t st = (cudaStream_t)stream;
    char *w = (char *)ws;
    SpMisc *misc = (SpMisc *)(w + L.off_misc);
    const long long *candptr = (const long long *)(w + L.off_candptr);
    const int *tmp = (const int *)(w + L.off_tmp);
    int cap = 0;
    CK(cudaMemcpyAsync(&cap, &misc->cap, sizeof cap, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    if (cap < 1) return op2g::fail(OP2G_ERR_INVALID, "op2g_sparsity_fill before op2g_sparsity_count");
    if (d->nrows == 0) return OP2G_OK;
    k_rows_copy<<<grid_for_rows(d->nrows), 256, 0, st>>>(d->nrows, candptr, tmp,
                                                         (const long long *)rowptr, colidx);
    CK(cudaGetLastError());
    return OP2G_OK;
}

}  // extern "C"

// ------------------------------------------------------------- matrices
namespace {

__device__ __forceinline__ long long find_col(const int64_t *rp, const int *ci, long long row,
                                              int col) {
    long long lo = rp[row], hi = rp[row + 1] - 1;
    while (lo <= hi) {
        const long long mid = (lo + hi) >> 1;
        const int c = ci[mid];
        if (c == col) return mid;
        if (c < col) lo = mid + 1;
        else hi = mid - 1;
    }
    return -1;
}

__global__ void k_zero_rows(op2g_bcsr m, const int *__restrict__ rows, long long n, double diag) {
    const int lane = threadIdx.x & 31;
    const long long w0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nw = ((long long)gridDim.x * blockDim.x) >> 5;
    const int bs = m.rdim * m.cdim;
    for (long long k = w0; k < n; k += nw) {
        const long long row = rows[k];
        if (row < 0 || row >= m.nrows * m.rdim) continue;
        const long long br = row / m.rdim;
        const int ri = (int)(row - br * m.rdim);
        const long long cb = row / m.cdim;
        const int cj0 = (int)(row - cb * m.cdim);
        for (long long q = m.rowptr[br] + lane; q < m.rowptr[br + 1]; q += 32)
            for (int cj = 0; cj < m.cdim; ++cj)
                m.values[q * bs + ri * m.cdim + cj] =
                    (m.colidx[q] == cb && cj == cj0) ? diag : 0.0;
    }
}

__global__ void k_set_diag(op2g_bcsr m, const int *__restrict__ rows, long long n, double diag,
                           int *err) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n; k += stride) {
        const long long row = rows[k];
        if (row < 0 || row >= m.nrows * m.rdim || row >= m.ncols * m.cdim) continue;
        const long long br = row / m.rdim, cb = row / m.cdim;
        const long long q = find_col(m.rowptr, m.colidx, br, (int)cb);
        if (q < 0) {
            if (err) atomicOr(err, OP2G_DEVERR_NEW_NONZERO);
            continue;
        }
        m.values[q * m.rdim * m.cdim + (row - br * m.rdim) * m.cdim + (row - cb * m.cdim)] = diag;
    }
}

// y = A x on block-CSR.  GB300 issues FP64 at 2 thread-instructions per
// clock per SM, so even a 1x1 product has as much FP64 time (one FMA per
// entry) as HBM time; every kernel below spends one FMA per entry and sums
// each row in a fixed order, so that repeated products are bitwise
// identical.
constexpr int SPMV_T = 256, SPMV_PER = 8, SPMV_TILE = SPMV_T * SPMV_PER;

// Blocks with more than 4 rows or columns (smaller ones run the lane kernel
// below): a block row holds hundreds of entries, so one thread per dof row
// would leave most lanes of a tile idle; instead S lanes share a dof row and
// the next tile's loads overlap the current sums.
//
// Work: a CTA takes slabs of NB consecutive block rows (grid-stride); NB is
// chosen from the mean row length so that a slab's entries fill about 90 %
// of one tile (SPMV_TILE entries, whole blocks), capped at one block row
// per thread.  A slab longer than a tile is walked in several tiles.
// Load: every thread issues up to SPMV_PER loads of values and column
// indices for the NEXT tile before summing the current one; the x gathers
// follow once the column indices are in; values and x are staged side by
// side in shared memory (double-buffered, one barrier per tile).
// Sum: S lanes (a power of two, S * NB * R <= SPMV_T) per dof row; lane s
// runs acc = fma(value, x, acc) over entries s, s + S, ... of its row in
// each tile of the slab (column order), and at the end of the slab the S
// partial sums are combined by butterfly shuffles.  NB and S depend only
// on the matrix.  RT/CT = block shape when known at compile time, 0 = from
// the descriptor.
template <int RT, int CT>
__global__ void __launch_bounds__(SPMV_T, 3)
    k_spmv_bsr(op2g_bcsr m, const double *__restrict__ x, double *__restrict__ y) {
    extern __shared__ double stage[];  // [2][2][QT * BS]: values | x, two buffers
    const int R = RT ? RT : m.rdim, C = CT ? CT : m.cdim;
    const int BS = R * C;
    const int QT = SPMV_TILE / BS;  // blocks per tile
    const int tid = threadIdx.x;
    int NB = SPMV_T / R;
    {
        const long long nnzb = __ldg(m.rowptr + m.nrows);
        if (nnzb > 0) {
            const long long fit = (long long)QT * m.nrows * 9 / (nnzb * 10);
            if (fit < NB) NB = fit < 1 ? 1 : (int)fit;
        }
    }
    int S = 1;
    while (S < 32 && 2 * S * NB * R <= SPMV_T) S <<= 1;
    const int grp = tid / S, lane_s = tid - grp * S;
    const bool has_row = grp < NB * R;
    const int lb = grp / R, ri = grp - lb * R;

    // tile cursor: slab [br0, brN) with entries [qs, qz) blocks; tile [qa, qe)
    long long br0 = blockIdx.x * (long long)NB;
    if (br0 >= m.nrows) return;
    const long long step = (long long)gridDim.x * NB;
    long long brN = br0 + NB < m.nrows ? br0 + NB : m.nrows;
    long long qz = __ldg(m.rowptr + brN);
    long long qa = __ldg(m.rowptr + br0);
    long long qe = qa + QT < qz ? qa + QT : qz;

    double v[SPMV_PER];
    int ci[SPMV_PER];
    auto issue = [&](long long qa_, long long qe_) {
        const int n = (int)((qe_ - qa_) * BS);
        const double *vals = m.values + qa_ * BS;
        const int *cols = m.colidx + qa_;
#pragma unroll
        for (int k = 0; k < SPMV_PER; ++k) {
            const int i = tid + k * SPMV_T;
            if (i < n) {
                v[k] = __ldg(vals + i);
                ci[k] = __ldg(cols + i / BS);
            }
        }
    };
    issue(qa, qe);

    // this thread's dof row in the current slab
    long long q0 = 0, q1 = 0;
    bool own = has_row && br0 + lb < brN;
    if (own) {
        q0 = __ldg(m.rowptr + br0 + lb);
        q1 = __ldg(m.rowptr + br0 + lb + 1);
    }
    double acc = 0.0;
    int buf = 0;
    for (;;) {
        // stage the tile whose loads are in flight
        {
            const int n = (int)((qe - qa) * BS);
            double *sv = stage + buf * 2 * QT * BS, *sx = sv + QT * BS;
            double xv[SPMV_PER];
#pragma unroll
            for (int k = 0; k < SPMV_PER; ++k) {
                const int i = tid + k * SPMV_T;
                if (i < n) {
                    const int w = i - (i / BS) * BS;
                    xv[k] = __ldg(x + ci[k] * C + (w - (w / C) * C));
                }
            }
#pragma unroll
            for (int k = 0; k < SPMV_PER; ++k) {
                const int i = tid + k * SPMV_T;
                if (i < n) {
                    sv[i] = v[k];
                    sx[i] = xv[k];
                }
            }
        }
        __syncthreads();  // tile staged; the buffer staged next was summed before this barrier
        // advance the cursor and put the next tile's loads in flight
        const long long cur_qa = qa, cur_qe = qe;
        const bool slab_end = qe >= qz;
        long long nbr0 = br0;
        bool more = true;
        if (!slab_end) {
            qa = qe;
            qe = qa + QT < qz ? qa + QT : qz;
        } else {
            nbr0 = br0 + step;
            more = nbr0 < m.nrows;
            if (more) {
                const long long nbrN = nbr0 + NB < m.nrows ? nbr0 + NB : m.nrows;
                qz = __ldg(m.rowptr + nbrN);
                qa = __ldg(m.rowptr + nbr0);
                qe = qa + QT < qz ? qa + QT : qz;
            }
        }
        if (more) issue(qa, qe);
        // sum the staged tile
        if (own) {
            const double *sv = stage + buf * 2 * QT * BS, *sx = sv + QT * BS;
            const long long s0 = q0 > cur_qa ? q0 : cur_qa, e0 = q1 < cur_qe ? q1 : cur_qe;
            const int len = (int)(e0 - s0) * C;
            const int base = (int)(s0 - cur_qa) * BS + ri * C;
            for (int j = lane_s; j < len; j += S) {
                const int dq = j / C;
                const int o = base + dq * BS + (j - dq * C);
                acc = fma(sv[o], sx[o], acc);
            }
        }
        if (slab_end) {
            for (int o = S >> 1; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
            if (own && lane_s == 0) y[(br0 + lb) * R + ri] = acc;
            acc = 0.0;
            if (!more) break;
            br0 = nbr0;
            brN = br0 + NB < m.nrows ? br0 + NB : m.nrows;
            own = has_row && br0 + lb < brN;
            if (own) {
                q0 = __ldg(m.rowptr + br0 + lb);
                q1 = __ldg(m.rowptr + br0 + lb + 1);
            }
        }
        buf ^= 1;
    }
}

// Any other block shape: a group of G lanes per dof row, lanes strided over
// the row's blocks.
template <int G>
__global__ void k_spmv_rows(op2g_bcsr m, const double *__restrict__ x, double *__restrict__ y) {
    constexpr int PER_WARP = 32 / G;
    const int lane = threadIdx.x & 31;
    const int sub = lane % G;
    const long long nr = m.nrows * m.rdim;
    const int bs = m.rdim * m.cdim;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long base = warp * PER_WARP; base < nr; base += nwarps * PER_WARP) {
        const long long row = base + lane / G;
        double acc = 0.0;
        if (row < nr) {
            const long long br = row / m.rdim;
            const int ri = (int)(row - br * m.rdim);
            for (long long q = m.rowptr[br] + sub; q < m.rowptr[br + 1]; q += G) {
                const long long c0 = (long long)m.colidx[q] * m.cdim;
                const double *v = m.values + q * bs + ri * m.cdim;
                for (int cj = 0; cj < m.cdim; ++cj) acc += v[cj] * x[c0 + cj];
            }
        }
#pragma unroll
        for (int o = G / 2; o > 0; o >>= 1) acc += __shfl_xor_sync(0xffffffffu, acc, o);
        if (row < nr && sub == 0) y[row] = acc;
    }
}

// y += A^T x (y zeroed by the caller) for blocks the lane kernel does not
// cover: a warp per block row walks its values with coalesced loads and adds
// each product into y with an atomic.
__global__ void k_spmv_t(op2g_bcsr m, const double *__restrict__ x, double *__restrict__ y) {
    const int lane = threadIdx.x & 31;
    const int bs = m.rdim * m.cdim;
    const long long warp = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long br = warp; br < m.nrows; br += nwarps) {
        const long long t1 = m.rowptr[br + 1] * bs;
        for (long long t = m.rowptr[br] * bs + lane; t < t1; t += 32) {
            const long long q = t / bs;
            const int w = (int)(t - q * bs);
            const int ri = w / m.cdim, cj = w - ri * m.cdim;
            atomicAdd(&y[(long long)m.colidx[q] * m.cdim + cj], m.values[t] * x[br * m.rdim + ri]);
        }
    }
}

unsigned grid_for(long long n, int bs) {
    long long g = (n + bs - 1) / bs;
    const long long cap = (long long)sms_of_current() * 16;
    if (g > cap) g = cap;
    return (unsigned)(g < 1 ? 1 : g);
}

// One lane per block row, so every FMA instruction is a full warp of useful
// work (the FP64 pipe's measure on this GPU) and no lanes' sums are
// combined.  A warp owns 32 consecutive block rows; each lane walks its own
// row K blocks at a time with their R C values and column indices in
// registers, and the next K blocks' loads are issued before the current
// ones' x gathers and FMAs.  A lane's blocks are contiguous, so its next
// loads hit the lines its last ones brought into L1.  Lanes past the end of
// their row skip the FMAs (their loads are of zeros and x[0..C)).  With TR
// the kernel adds A^T x into y instead: a lane holds its row's R values of
// x and scatters each block's C sums sum_i A[i][j] x_i with atomics.
// 3x3 and 2x2 blocks: K = 1, 3 CTAs of 256 threads per SM (68-72 registers);
// 1x1 (CSR): K = 4, 4 CTAs per SM.
// N doubles from p, VW per load through the read-only path (p aligned to
// 8 VW bytes; VW = 4 is one 256-bit load).
template <int N, int VW>
__device__ __forceinline__ void ld_doubles(double *v, const double *p) {
    if constexpr (VW == 4) {
#pragma unroll
        for (int k = 0; k < N / 4; ++k)
            asm("ld.global.nc.v4.f64 {%0, %1, %2, %3}, [%4];"
                : "=d"(v[4 * k]), "=d"(v[4 * k + 1]), "=d"(v[4 * k + 2]), "=d"(v[4 * k + 3])
                : "l"(p + 4 * k));
    } else if constexpr (VW == 2) {
#pragma unroll
        for (int k = 0; k < N / 2; ++k) {
            const double2 t = __ldg((const double2 *)p + k);
            v[2 * k] = t.x;
            v[2 * k + 1] = t.y;
        }
    } else {
#pragma unroll
        for (int e = 0; e < N; ++e) v[e] = __ldg(p + e);
    }
}

template <int R, int C, int K, int MINB, int VW, bool TR>
__global__ void __launch_bounds__(256, MINB)
    k_spmv_bsr_lane(op2g_bcsr m, const double *__restrict__ x, double *__restrict__ y) {
    constexpr int BS = R * C;
    const unsigned full = 0xffffffffu;
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    const long long nwarps = (long long)gridDim.x * (blockDim.x >> 5);
    for (long long r0 = ((long long)blockIdx.x * (blockDim.x >> 5) + wib) * 32; r0 < m.nrows;
         r0 += nwarps * 32) {
        const long long r = r0 + lane;
        long long q0 = 0, q1 = 0;
        if (r < m.nrows) {
            q0 = __ldg(m.rowptr + r);
            q1 = __ldg(m.rowptr + r + 1);
        }
        const int nsteps = ((int)__reduce_max_sync(full, (unsigned)(q1 - q0)) + K - 1) / K;
        const long long nvals = VW == -2 ? __ldg(m.rowptr + m.nrows) * BS : 0;
        double acc[R];
#pragma unroll
        for (int i = 0; i < R; ++i) acc[i] = 0.0;
        // y += A^T x: this row's x values, read once
        double xr[TR ? R : 1];
        if constexpr (TR) {
#pragma unroll
            for (int i = 0; i < R; ++i) xr[i] = r < m.nrows ? __ldg(x + r * R + i) : 0.0;
        }
        double v[K * BS];
        int col[K];
        // blocks [q, q + K) of this lane's row, zeros past its end
        auto load = [&](long long q) {
#pragma unroll
            for (int b = 0; b < K; ++b) {
                const bool ok = q + b < q1;
                col[b] = ok ? __ldg(m.colidx + q + b) : 0;
                if constexpr (VW == -2) {
                    // odd block size: the 16-byte pairs covering the block
                    // (it starts 8 bytes into a pair when its first element
                    // is odd); the last block, whose pairs could run one
                    // element past the array, one double at a time
                    const long long e0 = (q + b) * BS, a0 = e0 & ~1LL;
                    if (ok && a0 + BS + 1 <= nvals) {
                        double w[BS + 1];
                        ld_doubles<BS + 1, 2>(w, m.values + a0);
                        const bool odd = e0 & 1;
#pragma unroll
                        for (int e = 0; e < BS; ++e) v[b * BS + e] = odd ? w[e + 1] : w[e];
                    } else {
#pragma unroll
                        for (int e = 0; e < BS; ++e)
                            v[b * BS + e] = ok ? __ldg(m.values + e0 + e) : 0.0;
                    }
                } else if constexpr (VW == 1) {
#pragma unroll
                    for (int e = 0; e < BS; ++e)
                        v[b * BS + e] = ok ? __ldg(m.values + (q + b) * BS + e) : 0.0;
                } else if (ok) {
                    ld_doubles<BS, VW>(v + b * BS, m.values + (q + b) * BS);
                } else {
#pragma unroll
                    for (int e = 0; e < BS; ++e) v[b * BS + e] = 0.0;
                }
            }
        };
        if (nsteps > 0) load(q0);
        for (int k = 0; k < nsteps; ++k) {
            const long long qk = q0 + (long long)k * K;
            double cv[K * BS];
            int cc[K];
#pragma unroll
            for (int e = 0; e < K * BS; ++e) cv[e] = v[e];
#pragma unroll
            for (int b = 0; b < K; ++b) cc[b] = col[b];
            if (k + 1 < nsteps) load(qk + K);
            if constexpr (TR) {
                // block column j of y gets sum_i A[i][j] x_i (C atomics a block)
#pragma unroll
                for (int b = 0; b < K; ++b)
                    if (qk + b < q1) {
#pragma unroll
                        for (int j = 0; j < C; ++j) {
                            double t = 0.0;
#pragma unroll
                            for (int i = 0; i < R; ++i) t = fma(cv[b * BS + i * C + j], xr[i], t);
                            atomicAdd(y + (long long)cc[b] * C + j, t);
                        }
                    }
                continue;
            }
            double xv[K][C];
#pragma unroll
            for (int b = 0; b < K; ++b)
#pragma unroll
                for (int j = 0; j < C; ++j) xv[b][j] = __ldg(x + (long long)cc[b] * C + j);
#pragma unroll
            for (int b = 0; b < K; ++b)
                if (qk + b < q1) {
#pragma unroll
                    for (int i = 0; i < R; ++i)
#pragma unroll
                        for (int j = 0; j < C; ++j)
                            acc[i] = fma(cv[b * BS + i * C + j], xv[b][j], acc[i]);
                }
        }
        if (!TR && r < m.nrows) {
#pragma unroll
            for (int i = 0; i < R; ++i) y[r * R + i] = acc[i];
        }
    }
}

template <int R, int C, int K, int MINB, int VW, bool TR>
cudaError_t spmv_lane_go(cudaStream_t st, const op2g_bcsr &m, const double *x, double *y) {
    constexpr int T = 256;
    int dev = 0, occ = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_spmv_bsr_lane<R, C, K, MINB, VW, TR>,
                                                      T, 0);
    if (e != cudaSuccess) return e;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long warps = (m.nrows + 31) / 32;
    long long g = (long long)(occ > 0 ? occ : 1) * (sms > 0 ? sms : 1);
    const long long need = (warps + T / 32 - 1) / (T / 32);
    if (g > need) g = need;
    if (g < 1) g = 1;
    k_spmv_bsr_lane<R, C, K, MINB, VW, TR><<<(unsigned)g, T, 0, st>>>(m, x, y);
    return cudaGetLastError();
}

// Blocks of a multiple of 32 (16) bytes are 32- (16-) byte aligned when the
// values array is: they are then loaded 4 (2) doubles at a time.
template <int R, int C, int K, int MINB, bool TR = false>
cudaError_t spmv_lane_launch(cudaStream_t st, const op2g_bcsr &m, const double *x, double *y) {
    constexpr int BS = R * C;
    // 4 / 2: 256-bit / 16-byte loads; -2: odd blocks of 3 or more through
    // the 16-byte pairs that cover them; 1: one double at a time
    constexpr int VW = BS % 4 == 0 ? 4 : BS % 2 == 0 ? 2 : BS >= 3 ? -2 : 1;
    if constexpr (VW != 1) {
        const int al = VW == -2 ? 16 : 8 * VW;
        if ((uintptr_t)m.values % al == 0) return spmv_lane_go<R, C, K, MINB, VW, TR>(st, m, x, y);
    }
    return spmv_lane_go<R, C, K, MINB, 1, TR>(st, m, x, y);
}

// y += A^T x (y zeroed by the caller) for blocks up to 4 x 4; false when the
// shape has no lane kernel.
bool spmv_t_lane(cudaStream_t st, const op2g_bcsr &m, const double *x, double *y,
                 cudaError_t *e) {
    switch (m.rdim * 10 + m.cdim) {
        case 11: *e = spmv_lane_launch<1, 1, 4, 4, true>(st, m, x, y); return true;
        case 12: *e = spmv_lane_launch<1, 2, 2, 4, true>(st, m, x, y); return true;
        case 13: *e = spmv_lane_launch<1, 3, 2, 4, true>(st, m, x, y); return true;
        case 14: *e = spmv_lane_launch<1, 4, 2, 4, true>(st, m, x, y); return true;
        case 21: *e = spmv_lane_launch<2, 1, 2, 4, true>(st, m, x, y); return true;
        case 31: *e = spmv_lane_launch<3, 1, 2, 4, true>(st, m, x, y); return true;
        case 41: *e = spmv_lane_launch<4, 1, 2, 3, true>(st, m, x, y); return true;
        case 22: *e = spmv_lane_launch<2, 2, 1, 3, true>(st, m, x, y); return true;
        case 23: *e = spmv_lane_launch<2, 3, 1, 3, true>(st, m, x, y); return true;
        case 32: *e = spmv_lane_launch<3, 2, 1, 3, true>(st, m, x, y); return true;
        case 24: *e = spmv_lane_launch<2, 4, 1, 3, true>(st, m, x, y); return true;
        case 42: *e = spmv_lane_launch<4, 2, 1, 3, true>(st, m, x, y); return true;
        case 33: *e = spmv_lane_launch<3, 3, 1, 3, true>(st, m, x, y); return true;
        case 34: *e = spmv_lane_launch<3, 4, 1, 2, true>(st, m, x, y); return true;
        case 43: *e = spmv_lane_launch<4, 3, 1, 2, true>(st, m, x, y); return true;
        case 44: *e = spmv_lane_launch<4, 4, 1, 2, true>(st, m, x, y); return true;
    }
    return false;
}

// Launch k_spmv_bsr with more than the default 48 KB of dynamic shared
// memory (the attribute is set once per instantiation and size).
template <int RT, int CT>
cudaError_t spmv_launch(unsigned grid, size_t smem, cudaStream_t st, const op2g_bcsr &m,
                        const double *x, double *y) {
    static size_t granted = 0;
    if (smem > granted) {
        cudaError_t e = cudaFuncSetAttribute(k_spmv_bsr<RT, CT>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
        granted = smem;
    }
    k_spmv_bsr<RT, CT><<<grid, SPMV_T, smem, st>>>(m, x, y);
    return cudaGetLastError();
}

op2g_status check_bcsr(const op2g_bcsr *m) {
    if (!m || !m->rowptr || !m->values || m->rdim <= 0 || m->cdim <= 0 || m->nrows < 0)
        return op2g::fail(OP2G_ERR_INVALID, "bad block-CSR descriptor");
    return OP2G_OK;
}

}  // namespace

extern "C" {

op2g_status op2g_mat_zero_rows(const op2g_bcsr *m, const int32_t *rows, int64_t n, double diag,
                               void *stream) {
    op2g_status s = check_bcsr(m);
    if (s != OP2G_OK) return s;
    if (n <= 0) return OP2G_OK;
    k_zero_rows<<<grid_for(n * 32, 256), 256, 0, (cudaStream_t)stream>>>(*m, rows, n, diag);
    CK(cudaGetLastError());
    return OP2G_OK;
}

op2g_status op2g_mat_set_diagonal(const op2g_bcsr *m, const int32_t *rows, int64_t n, double diag,
                                  int32_t *err, void *stream) {
    op2g_status s = check_bcsr(m);
    if (s != OP2G_OK) return s;
    if (n <= 0) return OP2G_OK;
    k_set_diag<<<grid_for(n, 256), 256, 0, (cudaStream_t)stream>>>(*m, rows, n, diag, err);
    CK(cudaGetLastError());
    return OP2G_OK;
}

op2g_status op2g_mat_spmv(const op2g_bcsr *m, const double *x, double *y, int32_t transpose,
                          void *stream) {
    op2g_status s = check_bcsr(m);
    if (s != OP2G_OK) return s;
    const long long nr = m->nrows * m->rdim;
    if (nr <= 0) return OP2G_OK;
    cudaStream_t st = (cudaStream_t)stream;
    const int r = m->rdim, c = m->cdim;
    cudaError_t te = cudaSuccess;
    if (transpose) {
        // blocks up to 4 x 4: the lane kernel, C atomics per block (128^3
        // tet mesh: CSR 0.110 ms, 3x3 0.596 ms, against 0.590 / 1.692 ms for
        // a warp per row with an atomic per entry)
        if (m->ncols * c > INT_MAX || !spmv_t_lane(st, *m, x, y, &te))
            k_spmv_t<<<grid_for(m->nrows * 32, 256), 256, 0, st>>>(*m, x, y);
        CK(te);
    }
    else if (r > SPMV_T || r * c > SPMV_TILE || m->ncols * c > INT_MAX)
        k_spmv_rows<8><<<grid_for(nr * 8, 256), 256, 0, st>>>(*m, x, y);
    else if (r == 1 && c == 1)
        // tet mesh 128^3 (31.8 M entries): 0.090 ms, against 0.121 ms for a
        // CTA-tiled kernel staging values and x in shared memory
        CK((spmv_lane_launch<1, 1, 4, 4>(st, *m, x, y)));
    else {
        // two buffers of (SPMV_TILE / bs) * bs values and x entries
        const size_t smem = 4 * (size_t)(SPMV_TILE / (r * c)) * (r * c) * sizeof(double);
        const long long ctas = (m->nrows + SPMV_T / r - 1) / (SPMV_T / r);
        const unsigned g = grid_for(ctas * SPMV_T, SPMV_T);
        cudaError_t e;
        // Blocks up to 4 x 4: one lane per block row, K blocks per step, the
        // CTAs per SM its registers allow (measured on the 128^3 tet mesh,
        // 31.8 M blocks: 3.5-4x faster than the tiled kernel for every shape;
        // prism 3x3 matrix of 88.8 M blocks: 1.59 ms against 3.64 ms).
        switch (r * 10 + c) {
            case 12: e = spmv_lane_launch<1, 2, 2, 4>(st, *m, x, y); break;
            case 13: e = spmv_lane_launch<1, 3, 2, 4>(st, *m, x, y); break;
            case 14: e = spmv_lane_launch<1, 4, 2, 4>(st, *m, x, y); break;
            case 21: e = spmv_lane_launch<2, 1, 2, 4>(st, *m, x, y); break;
            case 31: e = spmv_lane_launch<3, 1, 2, 4>(st, *m, x, y); break;
            case 41: e = spmv_lane_launch<4, 1, 2, 3>(st, *m, x, y); break;
            case 22: e = spmv_lane_launch<2, 2, 1, 3>(st, *m, x, y); break;
            case 23: e = spmv_lane_launch<2, 3, 1, 3>(st, *m, x, y); break;
            case 32: e = spmv_lane_launch<3, 2, 1, 3>(st, *m, x, y); break;
            case 24: e = spmv_lane_launch<2, 4, 1, 3>(st, *m, x, y); break;
            case 42: e = spmv_lane_launch<4, 2, 1, 3>(st, *m, x, y); break;
            case 33: e = spmv_lane_launch<3, 3, 1, 3>(st, *m, x, y); break;
            case 34: e = spmv_lane_launch<3, 4, 1, 2>(st, *m, x, y); break;
            case 43: e = spmv_lane_launch<4, 3, 1, 2>(st, *m, x, y); break;
            case 44: e = spmv_lane_launch<4, 4, 1, 2>(st, *m, x, y); break;
            default: e = spmv_launch<0, 0>(g, smem, st, *m, x, y);
        }
        CK(e);
    }
    CK(cudaGetLastError());
    return OP2G_OK;
}

}  // extern "C"

// ------------------------------------------------------------- colouring
// Jones-Plassmann colouring on the implicit conflict graph "two entities
// conflict if they share a target through one of the maps".  Each round every
// uncoloured entity writes its priority (hash, id) into its targets with
// atomicMax; an entity that holds the maximum at all of its targets is a local
// maximum, so no two such entities share a target, and each takes the
// smallest colour absent from its targets' colour masks (first fit), then
// marks its colour there.  Rounds repeat until every entity is coloured.
namespace {

constexpr int CW = 4;  // 64-bit mask words per target -> at most 256 colours

struct ColDev {
    int nmaps;
    const int *maps[8];
    int arity[8];
    long long tsz[8];
    unsigned long long *tmax[8];
    unsigned long long *tmask[8];
};

__device__ __forceinline__ unsigned long long prio_of(long long c) {
    unsigned long long h = (unsigned long long)c * 0x9E3779B97F4A7C15ull;
    h ^= h >> 29;
    h *= 0xBF58476D1CE4E5B9ull;
    h ^= h >> 32;
    return (h << 32) | (unsigned long long)(c & 0xffffffffll);
}

__global__ void k_jp_prio(ColDev C, long long n, const int *__restrict__ colour) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += stride) {
        if (colour[c] >= 0) continue;
        const unsigned long long pr = prio_of(c);
        for (int k = 0; k < C.nmaps; ++k)
            for (int j = 0; j < C.arity[k]; ++j) {
                const int t = C.maps[k][c * C.arity[k] + j];
                if (t >= 0 && t < C.tsz[k]) atomicMax(&C.tmax[k][t], pr);
            }
    }
}

__global__ void k_jp_select(ColDev C, long long n, int *__restrict__ colour, int max_colours,
                            unsigned long long *__restrict__ remaining, int *__restrict__ err) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += stride) {
        if (colour[c] >= 0) continue;
        const unsigned long long pr = prio_of(c);
        bool top = true;
        unsigned long long used[CW] = {0, 0, 0, 0};
        for (int k = 0; k < C.nmaps && top; ++k)
            for (int j = 0; j < C.arity[k]; ++j) {
                const int t = C.maps[k][c * C.arity[k] + j];
                if (t < 0 || t >= C.tsz[k]) continue;
                if (C.tmax[k][t] != pr) {
                    top = false;
                    break;
                }
#pragma unroll
                for (int w = 0; w < CW; ++w) used[w] |= C.tmask[k][(long long)t * CW + w];
            }
        if (!top) {
            atomicAdd(remaining, 1ull);
            continue;
        }
        int col = -1;
        for (int w = 0; w < CW && col < 0; ++w)
            if (~used[w]) col = w * 64 + __ffsll((long long)~used[w]) - 1;
        if (col < 0 || col >= max_colours) {
            atomicOr(err, OP2G_DEVERR_CAPACITY);
            continue;
        }
        colour[c] = col;
        for (int k = 0; k < C.nmaps; ++k)
            for (int j = 0; j < C.arity[k]; ++j) {
                const int t = C.maps[k][c * C.arity[k] + j];
                if (t >= 0 && t < C.tsz[k])
                    atomicOr(&C.tmask[k][(long long)t * CW + col / 64], 1ull << (col % 64));
            }
    }
}

__global__ void k_col_hist(const int *__restrict__ colour, long long n, long long *__restrict__ cnt) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long c = blockIdx.x * (long long)blockDim.x + threadIdx.x; c < n; c += stride)
        atomicAdd((unsigned long long *)&cnt[colour[c]], 1ull);
}

// Stable placement: entity c goes to ptr[colour] + (number of entities of the
// same colour before c).  Each block handles a contiguous chunk; ranks within
// the chunk come from a per-colour running counter over the chunk in order.
__global__ void k_col_scatter(const int *__restrict__ colour, long long n, long long chunk,
                              const long long *__restrict__ chunk_base, int ncol,
                              int *__restrict__ order) {
    // chunk_base[b * ncol + k]: first slot of colour k for chunk b (exclusive scan)
    const long long b = blockIdx.x;
    const long long c0 = b * chunk, c1 = min(n, c0 + chunk);
    if (threadIdx.x != 0) return;
    extern __shared__ long long run[];
    for (int k = 0; k < ncol; ++k) run[k] = chunk_base[b * ncol + k];
    for (long long c = c0; c < c1; ++c) order[run[colour[c]]++] = (int)c;
}

__global__ void k_col_chunk_hist(const int *__restrict__ colour, long long n, long long chunk,
                                 int ncol, long long *__restrict__ h) {
    // h laid out colour-major: h[k * nchunks + b], so one exclusive scan gives
    // each (colour, chunk) its first slot in colour-then-entity order.
    const long long b = blockIdx.x;
    const long long nch = gridDim.x;
    const long long c0 = b * chunk, c1 = min(n, c0 + chunk);
    for (long long c = c0 + threadIdx.x; c < c1; c += blockDim.x)
        atomicAdd((unsigned long long *)&h[(long long)colour[c] * nch + b], 1ull);
}

__global__ void k_transpose_base(const long long *__restrict__ h, long long nch, int ncol,
                                 long long *__restrict__ base) {
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i >= nch * ncol) return;
    const long long b = i / ncol, k = i - b * ncol;
    base[i] = h[k * nch + b];
}

constexpr long long COL_CHUNK = 4096;

// Workspace layout of one colouring (the same for the caller's workspace and
// for the fixed array of op2g_colour_noalloc).  The histogram holds at least
// 257 entries: the colour count is read from its first 256 whatever ncells is.
size_t colour_layout(int64_t ncells, int32_t nmaps, const int64_t *target_size) {
    size_t off = 0;
    for (int k = 0; k < nmaps; ++k) {
        off = align256(off + sizeof(unsigned long long) * (size_t)target_size[k]);       // tmax
        off = align256(off + sizeof(unsigned long long) * CW * (size_t)target_size[k]);  // tmask
    }
    const long long nch = (ncells + COL_CHUNK - 1) / COL_CHUNK;
    const long long nh = (nch > 0 ? nch : 1) * 256 + 1;
    off = align256(off + sizeof(long long) * nh);                  // histogram
    off = align256(off + sizeof(long long) * nh);                  // transposed bases
    off = align256(off + sizeof(long long) * scan_tmp_elems(nh));  // scan temp
    off = align256(off + 64);                                      // counters
    return off;
}

// One colouring with its scratch at `ws` (colour_layout bytes, contents
// arbitrary: everything that must start at zero is cleared here).  Each
// Jones-Plassmann round reads its remaining count back to the host and
// synchronises `stream`; host-side arrays are on the stack.
op2g_status colour_run(int64_t ncells, int32_t nmaps, const int32_t *const *maps,
                       const int32_t *arity, const int64_t *target_size, int32_t max_colours,
                       void *ws, int32_t *colour, int32_t *order, int64_t *colour_ptr,
                       int32_t *ncolours, cudaStream_t st) {
    if (max_colours <= 0 || max_colours > 64 * CW)
        return op2g::fail(OP2G_ERR_INVALID, "max_colours must be in 1..256");
    if (!maps || !arity || !colour_ptr || (ncells > 0 && (!colour || !order)))
        return op2g::fail(OP2G_ERR_INVALID, "NULL argument");
    ColDev C;
    memset(&C, 0, sizeof C);
    C.nmaps = nmaps;
    char *w = (char *)ws;
    size_t off = 0;
    for (int k = 0; k < nmaps; ++k) {
        if (!maps[k] || arity[k] <= 0) return op2g::fail(OP2G_ERR_INVALID, "bad colouring map");
        C.maps[k] = maps[k];
        C.arity[k] = arity[k];
        C.tsz[k] = target_size[k];
        C.tmax[k] = (unsigned long long *)(w + off);
        off = align256(off + sizeof(unsigned long long) * (size_t)target_size[k]);
        C.tmask[k] = (unsigned long long *)(w + off);
        off = align256(off + sizeof(unsigned long long) * CW * (size_t)target_size[k]);
        CK(cudaMemsetAsync(C.tmask[k], 0, sizeof(unsigned long long) * CW * target_size[k], st));
    }
    const long long nch = (ncells + COL_CHUNK - 1) / COL_CHUNK;
    const long long nh = (nch > 0 ? nch : 1) * 256 + 1;
    long long *hist = (long long *)(w + off);
    off = align256(off + sizeof(long long) * nh);
    long long *base = (long long *)(w + off);
    off = align256(off + sizeof(long long) * nh);
    long long *scan = (long long *)(w + off);
    off = align256(off + sizeof(long long) * scan_tmp_elems(nh));
    unsigned long long *remaining = (unsigned long long *)(w + off);
    int *err = (int *)(remaining + 1);
    if (ncells > 0) CK(cudaMemsetAsync(colour, 0xff, sizeof(int) * ncells, st));
    CK(cudaMemsetAsync(err, 0, sizeof(int), st));
    const unsigned grid = grid_for(ncells, 256);
    unsigned long long left = (unsigned long long)ncells;
    int rounds = 0;
    while (left > 0) {
        if (++rounds > 100000) return op2g::fail(OP2G_ERR_TIMEOUT, "colouring did not converge");
        for (int k = 0; k < nmaps; ++k)
            CK(cudaMemsetAsync(C.tmax[k], 0, sizeof(unsigned long long) * target_size[k], st));
        CK(cudaMemsetAsync(remaining, 0, sizeof(unsigned long long), st));
        k_jp_prio<<<grid, 256, 0, st>>>(C, ncells, colour);
        k_jp_select<<<grid, 256, 0, st>>>(C, ncells, colour, max_colours, remaining, err);
        CK(cudaGetLastError());
        int herr = 0;
        CK(cudaMemcpyAsync(&left, remaining, sizeof left, cudaMemcpyDeviceToHost, st));
        CK(cudaMemcpyAsync(&herr, err, sizeof herr, cudaMemcpyDeviceToHost, st));
        CK(cudaStreamSynchronize(st));
        if (herr & OP2G_DEVERR_CAPACITY)
            return op2g::fail(OP2G_ERR_CAPACITY, "colouring needs more than max_colours colours");
    }
    // Number of colours = 1 + max colour; per-colour counts; stable order.
    long long hc[256];
    long long cp[64 * CW + 1];
    CK(cudaMemsetAsync(hist, 0, sizeof(long long) * 257, st));
    if (ncells > 0) k_col_hist<<<grid, 256, 0, st>>>(colour, ncells, hist);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(hc, hist, sizeof hc, cudaMemcpyDeviceToHost, st));
    CK(cudaStreamSynchronize(st));
    int ncol = 0;
    for (int k = 0; k < 256; ++k)
        if (hc[k]) ncol = k + 1;
    if (ncolours) *ncolours = ncol;
    cp[0] = 0;
    for (int k = 0; k < max_colours; ++k) cp[k + 1] = cp[k] + (k < ncol ? hc[k] : 0);
    CK(cudaMemcpyAsync(colour_ptr, cp, sizeof(long long) * (max_colours + 1),
                       cudaMemcpyHostToDevice, st));
    if (ncells > 0 && ncol > 0) {
        const long long nhist = nch * ncol;
        CK(cudaMemsetAsync(hist, 0, sizeof(long long) * (nhist + 1), st));
        k_col_chunk_hist<<<(unsigned)nch, 256, 0, st>>>(colour, ncells, COL_CHUNK, ncol, hist);
        CK(cudaGetLastError());
        op2g_status s = scan_exclusive(hist, nhist + 1, scan, st);
        if (s != OP2G_OK) return s;
        k_transpose_base<<<(unsigned)((nhist + 255) / 256), 256, 0, st>>>(hist, nch, ncol, base);
        k_col_scatter<<<(unsigned)nch, 32, sizeof(long long) * ncol, st>>>(colour, ncells, COL_CHUNK,
                                                                          base, ncol, order);
        CK(cudaGetLastError());
    }
    // the stack arrays hc / cp are read by the copies above: wait for them
    CK(cudaStreamSynchronize(st));
    return OP2G_OK;
}

}  // namespace

extern "C" {

op2g_status op2g_colour_workspace(int64_t ncells, int32_t nmaps, const int64_t *target_size,
                                  size_t *bytes) {
    if (nmaps <= 0 || nmaps > 8 || !target_size || ncells < 0)
        return op2g::fail(OP2G_ERR_INVALID, "colouring takes 1..8 maps");
    for (int k = 0; k < nmaps; ++k)
        if (target_size[k] < 0) return op2g::fail(OP2G_ERR_INVALID, "negative target size");
    const size_t off = colour_layout(ncells, nmaps, target_size);
    if (bytes) *bytes = off;
    return OP2G_OK;
}

op2g_status op2g_colour(int64_t ncells, int32_t nmaps, const int32_t *const *maps,
                        const int32_t *arity, const int64_t *target_size, int32_t max_colours,
                        void *ws, size_t ws_bytes, int32_t *colour, int32_t *order,
                        int64_t *colour_ptr, int32_t *ncolours, void *stream) {
    size_t need = 0;
    op2g_status s = op2g_colour_workspace(ncells, nmaps, target_size, &need);
    if (s != OP2G_OK) return s;
    if (!ws || ws_bytes < need) return op2g::fail(OP2G_ERR_INVALID, "workspace too small");
    return colour_run(ncells, nmaps, maps, arity, target_size, max_colours, ws, colour, order,
                      colour_ptr, ncolours, (cudaStream_t)stream);
}

}  // extern "C"

// ------------------------------------------------- colouring without allocation
// For callers that cannot allocate device memory: a host embedding the
// library in a process whose device memory belongs to another allocator (a
// framework's caching allocator, a memory pool sized up front), or a runtime
// that forbids cudaMalloc after start-up.  op2g_colour_noalloc runs the same
// colouring (colour_run) with its scratch in a fixed device array of this
// file instead of a caller-provided workspace; the caller still passes every
// input and output.  Like op2g_colour it synchronises the stream every
// Jones-Plassmann round.
namespace {

// Every GPU that loads the library holds this array until the process exits.
__device__ __align__(256) unsigned char g_colour_scratch[OP2G_COLOUR_NOALLOC_SCRATCH_BYTES];

std::mutex g_colour_scratch_mu;
void *g_colour_scratch_addr[OP2G_NOALLOC_MAX_DEVICES];  // device address, per device

// Device address of g_colour_scratch on the current device.  The host-side
// name of a __device__ array is only a stand-in: the address has to come from
// cudaGetSymbolAddress, done once per device with that device current.
op2g_status colour_scratch(void **out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return op2g::cuda_fail(e, "cudaGetDevice");
    if (dev < 0 || dev >= OP2G_NOALLOC_MAX_DEVICES)
        return op2g::fail(OP2G_ERR_UNSUPPORTED, "device index above OP2G_NOALLOC_MAX_DEVICES");
    std::lock_guard<std::mutex> g(g_colour_scratch_mu);
    if (!g_colour_scratch_addr[dev]) {
        void *p = nullptr;
        e = cudaGetSymbolAddress(&p, g_colour_scratch);
        if (e != cudaSuccess) return op2g::cuda_fail(e, "cudaGetSymbolAddress(g_colour_scratch)");
        g_colour_scratch_addr[dev] = p;
    }
    *out = g_colour_scratch_addr[dev];
    return OP2G_OK;
}

}  // namespace

extern "C" op2g_status op2g_colour_noalloc(int64_t ncells, int32_t nmaps,
                                           const int32_t *const *maps, const int32_t *arity,
                                           const int64_t *target_size, int32_t max_colours,
                                           int32_t *colour, int32_t *order, int64_t *colour_ptr,
                                           int32_t *ncolours, void *stream) {
    size_t need = 0;
    op2g_status s = op2g_colour_workspace(ncells, nmaps, target_size, &need);
    if (s != OP2G_OK) return s;
    if (need > (size_t)OP2G_COLOUR_NOALLOC_SCRATCH_BYTES)
        return op2g::fail(OP2G_ERR_CAPACITY,
                          "op2g_colour_noalloc: problem needs " + std::to_string(need) +
                              " bytes of scratch, above the fixed " +
                              std::to_string((long long)OP2G_COLOUR_NOALLOC_SCRATCH_BYTES) +
                              " (use op2g_colour with a workspace)");
    void *ws = nullptr;
    s = colour_scratch(&ws);
    if (s != OP2G_OK) return s;
    return colour_run(ncells, nmaps, maps, arity, target_size, max_colours, ws, colour, order,
                      colour_ptr, ncolours, (cudaStream_t)stream);
}

// ---------------------------------------------------------------- probe
// FP64 FMA throughput: every thread runs CHAINS independent FMA chains
// (x = x * a + b), so each warp always has CHAINS instructions ready while
// earlier ones are in flight; the grid holds 8 CTAs of 256 threads per SM.
namespace {
constexpr int CHAINS = 16;
__device__ double g_dfma_sink;
__global__ void __launch_bounds__(256) k_dfma(int iters, double a, double b) {
    double x[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = threadIdx.x * 1e-9 + c;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) x[c] = fma(x[c], a, b);
    }
    double s = 0.0;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += x[c];
    if (s == 1234.5678) g_dfma_sink = s;  // keeps the chains alive
}
}  // namespace

extern "C" op2g_status op2g_probe_fp64_peak(double *flops, void *stream) {
    if (!flops) return op2g::fail(OP2G_ERR_INVALID, "NULL output");
    cudaStream_t st = (cudaStream_t)stream;
    const int sms = sms_of_current();
    const int blocks = sms * 8, threads = 256, iters = 2048;
    cudaEvent_t e0, e1;
    CK(cudaEventCreate(&e0));
    CK(cudaEventCreate(&e1));
    k_dfma<<<blocks, threads, 0, st>>>(iters, 0.999999, 1e-7);  // warm-up
    float best = 1e30f;
    for (int rep = 0; rep < 5; ++rep) {
        CK(cudaEventRecord(e0, st));
        k_dfma<<<blocks, threads, 0, st>>>(iters, 0.999999, 1e-7);
        CK(cudaEventRecord(e1, st));
        CK(cudaEventSynchronize(e1));
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, e0, e1));
        if (ms < best) best = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    *flops = 2.0 * CHAINS * (double)iters * (double)blocks * threads / (best * 1e-3);
    return OP2G_OK;
}
