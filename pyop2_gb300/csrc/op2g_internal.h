// op2g_internal.h -- shared declarations of libop2g's C++ translation units.
#pragma once

#include <string>
#include <utility>
#include <vector>

#include "../../include/op2g.h"

namespace op2g {

// Thread-local error reporting behind op2g_last_error().
op2g_status fail(op2g_status code, const std::string &msg);
op2g_status cuda_fail(int err, const char *what);

struct MapInfo {
    int kind = OP2G_MAP_PLAIN;
    int arity = 0;
    int base = -1;
    int ncomposed = 0;
    int composed[OP2G_MAX_COMPOSED] = {0};
    std::vector<int> offset, offset_quotient, permutation;
};

struct ArgInfo {
    op2g_arg_desc d;
    int slot = 0;  // first device-pointer slot
};

// Everything that determines the generated code of one wrapper.
struct Signature {
    std::string user_src, kernel_name;
    op2g_loop_desc loop;
    std::vector<ArgInfo> args;
    std::vector<MapInfo> maps;
    int nptrs = 0;          // argument slots + one slot per map
    int map_slot0 = 0;      // first map slot
    int block_size = 256;
    int map_slot(int m) const { return map_slot0 + m; }
};

std::string validate_signature(const Signature &S);
// The wrapper's source; *cells_per_thread (may be NULL) receives the
// iterations a thread runs per sweep step in it.  With align_hints the
// direct arguments of aligned_direct_args are declared aligned (the variant
// launched only when their pointers are).
std::string generate_source(const Signature &S, int *cells_per_thread = nullptr,
                            bool align_hints = false);
// Direct Dat arguments whose rows are a multiple of 16 bytes, as (pointer
// slot, row alignment in bytes: 16 or 32); empty for staged wrappers.
std::vector<std::pair<int, int>> aligned_direct_args(const Signature &S);
int direct_row_alignment(const Signature &S, size_t a);
// Staged wrappers (OP2G_SCATTER_STAGED): per argument the plain map whose
// staging plan it uses, or -1; and the dynamic shared memory they take.
std::vector<int> staged_args(const Signature &S);
std::vector<bool> staged_direct(const Signature &S);
size_t staged_smem_bytes(const Signature &S, int64_t block, const int32_t *max_unique);

// Exclusive in-place prefix sum of d[0..n) on `st` (device memory); tmp holds
// scan_tmp_elems(n) elements (op2g_kernels.cu).
size_t scan_tmp_elems(long long n);
op2g_status scan_exclusive(long long *d, long long n, long long *tmp, struct CUstream_st *st);

// Text of op2g_device.cuh, embedded at build time.
extern const char *const device_header_src;

}  // namespace op2g
