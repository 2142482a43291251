// op2g_codegen.cpp -- writes the CUDA wrapper for one par_loop signature.
//
// The reference generates, per (local kernel, argument signature), a C loop
// that packs each argument, calls the kernel and unpacks
// (pyop2/codegen/builder.py:683-989, lowered by rep2loopy.py).  Here the same
// contract is written directly as CUDA: one thread per iteration entity (or
// per (entity, layer) for constant-layer extrusion), packs in registers, the
// user's kernel inlined as a __device__ function, and conflict handling for
// INC/MIN/MAX by atomics, warp aggregation, or plain stores when the caller
// iterates one colour at a time.
#include "op2g_internal.h"

#include <cctype>
#include <sstream>

namespace op2g {

static const char *ctype_of(int dt) {
    switch (dt) {
        case OP2G_F64: return "double";
        case OP2G_F32: return "float";
        case OP2G_I32: return "int";
        case OP2G_U32: return "unsigned";
        case OP2G_I64: return "long long";
        case OP2G_U64: return "unsigned long long";
        case OP2G_I16: return "short";
        case OP2G_U16: return "unsigned short";
        case OP2G_I8: return "signed char";
        case OP2G_U8: return "unsigned char";
    }
    return nullptr;
}

static bool atomic_capable(int dt) {
    return dt == OP2G_F64 || dt == OP2G_F32 || dt == OP2G_I32 || dt == OP2G_U32 ||
           dt == OP2G_I64 || dt == OP2G_U64;
}

// Strip `#include <...>` lines of C system headers: NVRTC has no host system
// headers, and the device math library and fixed-width integer types they
// would declare are provided by NVRTC and op2g_device.cuh.  Any other include
// is kept (and fails to compile if it cannot be found, as it should).
static std::string strip_system_includes(const std::string &src) {
    static const char *known[] = {"math.h", "stdio.h", "stdlib.h", "string.h", "stdint.h",
                                  "stdbool.h", "complex.h", "petsc.h", "inttypes.h",
                                  "float.h", "limits.h", "cmath", "cstdio", "cstdlib",
                                  "cstring", "cstdint", "algorithm"};
    std::istringstream in(src);
    std::ostringstream out;
    std::string line;
    while (std::getline(in, line)) {
        size_t p = line.find_first_not_of(" \t");
        bool drop = false;
        if (p != std::string::npos && line[p] == '#') {
            size_t q = line.find("include", p);
            if (q != std::string::npos) {
                size_t lt = line.find('<', q), gt = line.find('>', q);
                if (lt != std::string::npos && gt != std::string::npos && gt > lt) {
                    std::string h = line.substr(lt + 1, gt - lt - 1);
                    for (const char *k : known)
                        if (h == k) drop = true;
                }
            }
        }
        out << (drop ? std::string("// (system include supplied by op2g) ") + line : line)
            << "\n";
    }
    return out.str();
}

// True when the user kernel is declared with an empty parameter list,
// `name()` or `name(void)`.  In C (the reference compiles kernels as C) an
// empty list leaves the parameters unspecified, so the wrapper may pass the
// packs anyway; in CUDA C++ it means "no parameters", so the call is then
// made without arguments.
static bool declared_without_parameters(const std::string &src, const std::string &name) {
    auto is_ident = [](char c) { return std::isalnum((unsigned char)c) || c == '_'; };
    for (size_t p = src.find(name); p != std::string::npos; p = src.find(name, p + 1)) {
        if (p > 0 && is_ident(src[p - 1])) continue;
        size_t q = p + name.size();
        if (q < src.size() && is_ident(src[q])) continue;
        while (q < src.size() && std::isspace((unsigned char)src[q])) ++q;
        if (q >= src.size() || src[q] != '(') continue;
        ++q;
        while (q < src.size() && std::isspace((unsigned char)src[q])) ++q;
        if (src.compare(q, 4, "void") == 0 && (q + 4 >= src.size() || !is_ident(src[q + 4]))) {
            q += 4;
            while (q < src.size() && std::isspace((unsigned char)src[q])) ++q;
        }
        if (q < src.size() && src[q] == ')') return true;
    }
    return false;
}

// Starting value of an INC accumulator (Global, Dat and Mat packs; the
// reference zero-fills them, pyop2/codegen/builder.py:271-274, 353-356,
// 538-541).  For floating types it is -0.0, the exact identity of IEEE
// addition: -0.0 + w == w for every w, so the compiler drops the kernel's
// first `+=` into each entry (a DADD per entry: 4 of the P1 tet action's 64
// FP64 instructions per cell), whereas +0.0 + w turns w = -0.0 into +0.0.
// The scattered value then differs from the reference's only when it is
// -0.0, and the sum it is added to only when that sum is also -0.0 (-0.0
// here, +0.0 in the reference; the two compare equal).
static std::string inc_zero(int dt) {
    if (dt == OP2G_F64) return "(-0.0)";
    if (dt == OP2G_F32) return "(-0.0f)";
    return std::string("(") + ctype_of(dt) + ")0";
}

static size_t elt_size(int dt) {
    switch (dt) {
        case OP2G_F64: case OP2G_I64: case OP2G_U64: return 8;
        case OP2G_F32: case OP2G_I32: case OP2G_U32: return 4;
        case OP2G_I16: case OP2G_U16: return 2;
        default: return 1;
    }
}

// ---------------------------------------------------------------------------
// Which arguments a staged wrapper (OP2G_SCATTER_STAGED) stages in shared
// memory: Dat arguments (not parts of a mixed argument) through a plain map
// or a permuted one, READ when no argument of the loop writes a Dat that a
// READ argument reads (staged values are read once per partition), and INC
// with an element type shared-memory atomics support.  Entry a is the plain
// map whose plan the argument uses, or -1.  Non-extruded, non-indexed loops
// only; an empty result means the wrapper runs as OP2G_SCATTER_ATOMIC.
std::vector<int> staged_args(const Signature &S) {
    std::vector<int> st(S.args.size(), -1);
    if (S.loop.scatter != OP2G_SCATTER_STAGED || S.loop.extruded || S.loop.indexed) return st;
    for (size_t a = 0; a < S.args.size(); ++a) {
        const op2g_arg_desc &d = S.args[a].d;
        if (d.kind != OP2G_ARG_DAT || d.map < 0 || d.group != 0) continue;
        const MapInfo &mi = S.maps[d.map];
        int root = -1;
        if (mi.kind == OP2G_MAP_PLAIN) root = d.map;
        else if (mi.kind == OP2G_MAP_PERMUTED) root = mi.base;
        if (root < 0) continue;
        const size_t e = elt_size(d.dtype);
        const bool inc_ok = d.access == OP2G_INC &&
                            (d.dtype == OP2G_F64 || d.dtype == OP2G_F32 || d.dtype == OP2G_I32 ||
                             d.dtype == OP2G_U32 || d.dtype == OP2G_U64 || d.dtype == OP2G_I64);
        const bool read_ok = d.access == OP2G_READ && S.loop.nc_reads && (e == 4 || e == 8);
        if (!inc_ok && !read_ok) continue;
        st[a] = root;
    }
    return st;
}

// Direct READ arguments a staged wrapper fetches ahead into shared memory
// (4- or 8-byte elements, not parts of a mixed argument); only when the
// wrapper stages at least one argument.
std::vector<bool> staged_direct(const Signature &S) {
    std::vector<bool> out(S.args.size(), false);
    std::vector<int> st = staged_args(S);
    bool any = false;
    for (int r : st) any = any || r >= 0;
    if (!any) return out;
    for (size_t a = 0; a < S.args.size(); ++a) {
        const op2g_arg_desc &d = S.args[a].d;
        const size_t e = elt_size(d.dtype);
        out[a] = d.kind == OP2G_ARG_DAT && d.map < 0 && d.access == OP2G_READ && d.group == 0 &&
                 (e == 4 || e == 8);
    }
    return out;
}

// Bytes of dynamic shared memory a staged wrapper takes for partitions of
// `block` iterations whose largest distinct-target counts are max_unique[m]
// -- the layout the generated code computes, every region rounded up to 16
// bytes: per staged map, three plan buffers (target list, run offsets, the
// partition's slots) and the slot -> target table; per staged READ argument
// two value buffers (one value per target); per staged INC argument one
// value per slot; per fetched direct argument two buffers of the
// partition's values.
size_t staged_smem_bytes(const Signature &S, int64_t block, const int32_t *max_unique) {
    std::vector<int> st = staged_args(S);
    std::vector<bool> dr = staged_direct(S);
    auto r16 = [](size_t x) { return (x + 15) & ~(size_t)15; };
    size_t bytes = 0;
    std::vector<bool> seen(S.maps.size(), false);
    for (size_t a = 0; a < st.size(); ++a)
        if (st[a] >= 0) seen[st[a]] = true;
    for (size_t m = 0; m < S.maps.size(); ++m)
        if (seen[m]) {
            const size_t seg = ((size_t)max_unique[m] + 1 + 7) / 8 * 8;
            const size_t slots = (size_t)block * S.maps[m].arity;
            bytes += 3 * (r16(seg * 4) + r16(seg * 2) + r16(slots * 2)) + r16(slots * 2);
        }
    for (size_t a = 0; a < st.size(); ++a) {
        const op2g_arg_desc &d = S.args[a].d;
        const size_t e = elt_size(d.dtype);
        if (st[a] >= 0 && d.access == OP2G_READ)
            bytes += 2 * r16((size_t)max_unique[st[a]] * d.dim * e);
        else if (st[a] >= 0)
            bytes += r16((size_t)block * S.maps[st[a]].arity * d.dim * e);
        else if (dr[a])
            bytes += 2 * r16((size_t)block * d.dim * e);
    }
    return bytes;
}

struct Gen {
    const Signature &S;
    std::ostringstream o;
    int nf = 1;  // 2 for ON_INTERIOR_FACETS (packs span two cells of a column)

    // Kernel-parameter layout.  Consecutive arguments with one group id are
    // one kernel parameter: a MixedDat's component packs concatenated
    // (pyop2/codegen/builder.py:413-498), or a mixed Mat's blocks as
    // sub-blocks of one element matrix (pyop2/codegen/builder.py:609-680).
    std::vector<int> first;   // first argument of the parameter
    std::vector<int> poff;    // DAT: offset of this component's pack
    std::vector<int> roff, coff, rstride;  // MAT: sub-block origin, element-matrix width
    std::vector<int> psize;   // at first: size of the parameter's pack
    bool has_groups = false;

    // Staging (OP2G_SCATTER_STAGED): per argument the plain map of its plan
    // or -1; per map whether the wrapper loads its plan; set while the
    // staged run function is written.
    std::vector<int> st_arg;
    std::vector<bool> st_map, st_dir;
    bool any_staged = false, staging = false;
    // Several cells per thread per sweep step: iterations past the end run
    // on a clamped (valid) iteration and only their unpack is skipped, so the
    // cells' gathers and arithmetic can be interleaved by the compiler.
    bool guard_unpack = false;
    int cells_per_thread = 1;  // what the sweep loop was generated with
    // The variant for aligned direct arguments (aligned_direct_args).
    bool align_hints = false;

    explicit Gen(const Signature &s) : S(s) {
        nf = (S.loop.extruded && S.loop.iteration_region == OP2G_ON_INTERIOR_FACETS) ? 2 : 1;
        layout();
        st_arg = staged_args(S);
        st_dir = staged_direct(S);
        st_map.assign(S.maps.size(), false);
        for (int r : st_arg)
            if (r >= 0) {
                st_map[r] = true;
                any_staged = true;
            }
    }

    // Elements between consecutive entities' values of a Dat argument.
    int gstride(size_t a) const {
        const op2g_arg_desc &d = S.args[a].d;
        return d.stride > 0 ? d.stride : d.dim;
    }

    int dat_pack(size_t a) const {
        const op2g_arg_desc &d = S.args[a].d;
        return d.map >= 0 ? nf * S.maps[d.map].arity * d.dim : d.dim;
    }
    int mat_rows(size_t a) const {
        const op2g_arg_desc &d = S.args[a].d;
        return nf * S.maps[d.map].arity * d.rdim;
    }
    int mat_cols(size_t a) const {
        const op2g_arg_desc &d = S.args[a].d;
        return nf * S.maps[d.cmap].arity * d.cdim;
    }

    // Shared-memory staging of INC contributions (OP2G_SCATTER_SHARED):
    // per INC-through-a-map argument, a table of 2 x (contributions per CTA)
    // slots rounded to a power of two, shrunk to fit 40 KB of static shared
    // memory in total; an argument that does not fit keeps global atomics.
    std::vector<int> shared_ts;
    bool any_shared = false;

    void plan_shared(bool on) {
        shared_ts.assign(S.args.size(), 0);
        any_shared = false;
        if (!on) return;
        size_t budget = 40 * 1024;
        for (size_t a = 0; a < S.args.size(); ++a) {
            const op2g_arg_desc &d = S.args[a].d;
            if (d.kind != OP2G_ARG_DAT || d.map < 0 || d.access != OP2G_INC) continue;
            if (!atomic_capable(d.dtype)) continue;
            const int contrib = S.block_size * nf * S.maps[d.map].arity;
            int ts = 1;
            while (ts < 2 * contrib) ts <<= 1;
            const size_t elt = d.dtype == OP2G_F64 || d.dtype == OP2G_I64 || d.dtype == OP2G_U64 ? 8 : 4;
            auto bytes = [&](int t) { return (size_t)t * (8 + elt * d.dim) + 8; };
            while (ts > contrib && bytes(ts) > budget) ts >>= 1;
            if (ts < contrib || bytes(ts) > budget) continue;
            shared_ts[a] = ts;
            budget -= bytes(ts);
            any_shared = true;
        }
    }

    void layout() {
        const size_t n = S.args.size();
        first.assign(n, 0);
        poff.assign(n, 0);
        roff.assign(n, 0);
        coff.assign(n, 0);
        rstride.assign(n, 0);
        psize.assign(n, 0);
        for (size_t a = 0; a < n;) {
            const op2g_arg_desc &d0 = S.args[a].d;
            size_t b = a + 1;
            if (d0.group > 0) {
                has_groups = true;
                while (b < n && S.args[b].d.group == d0.group) ++b;
            }
            for (size_t k = a; k < b; ++k) first[k] = (int)a;
            if (d0.kind == OP2G_ARG_DAT) {
                int off = 0;
                for (size_t k = a; k < b; ++k) {
                    poff[k] = off;
                    off += dat_pack(k);
                }
                psize[a] = off;
            } else if (d0.kind == OP2G_ARG_MAT) {
                const int C = d0.group > 0 ? d0.group_cols : 1;
                const int R = (int)(b - a) / C;
                std::vector<int> co(C), ro(R);
                int tc = 0, tr = 0;
                for (int j = 0; j < C; ++j) { co[j] = tc; tc += mat_cols(a + j); }
                for (int i = 0; i < R; ++i) { ro[i] = tr; tr += mat_rows(a + (size_t)i * C); }
                for (size_t k = a; k < b; ++k) {
                    roff[k] = ro[(k - a) / C];
                    coff[k] = co[(k - a) % C];
                    rstride[k] = tc;
                }
                psize[a] = tr * tc;
            }
            a = b;
        }
    }

    // Map used for the outermost indexing of map m (PERMUTED -> its base).
    int root_of(int m) const {
        const MapInfo &mi = S.maps[m];
        return mi.kind == OP2G_MAP_PERMUTED ? mi.base : m;
    }

    // Names of the per-iteration base rows.
    std::string base_row(int m) const { return "mv" + std::to_string(m); }
    std::string idx_arr(int m, int f) const {
        return "mi" + std::to_string(m) + "_" + std::to_string(f);
    }

    void emit_constants() {
        for (size_t m = 0; m < S.maps.size(); ++m) {
            const MapInfo &mi = S.maps[m];
            auto arr = [&](const char *nm, const std::vector<int> &v) {
                o << "__device__ const int op2g_" << nm << m << "[" << v.size() << "] = {";
                for (size_t i = 0; i < v.size(); ++i) o << (i ? ", " : "") << v[i];
                o << "};\n";
            };
            if (!mi.offset.empty()) arr("off", mi.offset);
            if (!mi.offset_quotient.empty()) arr("offq", mi.offset_quotient);
            if (!mi.permutation.empty()) arr("perm", mi.permutation);
        }
    }

    // Which maps need per-iteration index arrays.
    std::vector<bool> used_maps() const {
        std::vector<bool> used(S.maps.size(), false);
        for (const ArgInfo &a : S.args) {
            if (a.d.kind == OP2G_ARG_DAT && a.d.map >= 0) used[a.d.map] = true;
            if (a.d.kind == OP2G_ARG_MAT) {
                used[a.d.map] = true;
                used[a.d.cmap] = true;
            }
        }
        return used;
    }

    // Emit loading of the base row for plain map m at entity expression `ent`
    // into `dst` (declared when `declare`).  Maps are read-only during a
    // launch, so rows go through the non-coherent path, as 16- or 8-byte
    // vectors when the arity allows (alignment is checked at launch).
    void emit_plain_row(int m, const std::string &ent, const std::string &ind,
                        std::string dst = "", bool declare = true) {
        const MapInfo &mi = S.maps[m];
        if (dst.empty()) dst = base_row(m);
        if (declare) o << ind << "int " << dst << "[" << mi.arity << "];\n";
        o << ind << "{ const int *r_ = (const int *)p.ptr[" << S.map_slot(m) << "] + (" << ent
          << ") * " << mi.arity << ";\n";
        if (mi.arity % 4 == 0) {
            for (int q = 0; q < mi.arity / 4; ++q)
                o << ind << "  { const int4 v_ = __ldg((const int4 *)r_ + " << q << "); " << dst
                  << "[" << 4 * q << "] = v_.x; " << dst << "[" << 4 * q + 1 << "] = v_.y; " << dst
                  << "[" << 4 * q + 2 << "] = v_.z; " << dst << "[" << 4 * q + 3 << "] = v_.w; }\n";
        } else if (mi.arity % 2 == 0) {
            for (int q = 0; q < mi.arity / 2; ++q)
                o << ind << "  { const int2 v_ = __ldg((const int2 *)r_ + " << q << "); " << dst
                  << "[" << 2 * q << "] = v_.x; " << dst << "[" << 2 * q + 1 << "] = v_.y; }\n";
        } else {
            o << ind << "#pragma unroll\n";
            o << ind << "  for (int i = 0; i < " << mi.arity << "; ++i) " << dst
              << "[i] = __ldg(r_ + i);\n";
        }
        o << ind << "}\n";
    }

    // Plain maps whose rows an iteration loads (directly or for a permuted map).
    std::vector<bool> row_maps() const {
        std::vector<bool> used = used_maps();
        std::vector<bool> need(S.maps.size(), false);
        for (size_t m = 0; m < S.maps.size(); ++m) {
            if (!used[m]) continue;
            const MapInfo &mi = S.maps[m];
            if (mi.kind == OP2G_MAP_PLAIN) need[m] = true;
            else if (mi.kind == OP2G_MAP_PERMUTED) need[mi.base] = true;
        }
        return need;
    }

    // Emit index arrays mi<m>_<f>[arity] for map m (after base rows exist).
    void emit_index_arrays(int m, const std::string &ind) {
        const MapInfo &mi = S.maps[m];
        // Resolve: outermost plain map supplying the values, and the row it reads.
        std::string rowname;
        int src = m;
        if (mi.kind == OP2G_MAP_PLAIN) {
            rowname = base_row(m);
        } else if (mi.kind == OP2G_MAP_PERMUTED) {
            rowname = base_row(mi.base);
            src = mi.base;
        } else {  // COMPOSED: chain maps_[k-1] .. maps_[1] (arity 1), then maps_[0]
            const int outer = mi.composed[0];
            const MapInfo &om = S.maps[outer];
            int oroot = outer;
            std::string operm;
            if (om.kind == OP2G_MAP_PERMUTED) {
                oroot = om.base;
                operm = "op2g_perm" + std::to_string(outer);
            }
            o << ind << "int " << base_row(m) << "[" << mi.arity << "];\n";
            o << ind << "{ long long c_ = n;\n";
            for (int k = mi.ncomposed - 1; k >= 1; --k) {
                int cm = mi.composed[k];
                int croot = root_of(cm);
                o << ind << "  if (c_ >= 0) c_ = ((const int *)p.ptr[" << S.map_slot(croot)
                  << "])[c_ * " << S.maps[croot].arity << "];\n";
            }
            o << ind << "#pragma unroll\n";
            o << ind << "  for (int i = 0; i < " << mi.arity << "; ++i) " << base_row(m)
              << "[i] = c_ >= 0 ? ((const int *)p.ptr[" << S.map_slot(oroot) << "])[c_ * "
              << S.maps[oroot].arity << " + " << (operm.empty() ? "i" : operm + "[i]")
              << "] : -1; }\n";
            rowname = base_row(m);
            src = outer;  // offsets come from maps_[0] (pyop2/types/map.py:271)
            if (om.kind == OP2G_MAP_PERMUTED) src = om.base;
        }
        const MapInfo &sm = S.maps[src];
        const bool perm = (mi.kind == OP2G_MAP_PERMUTED);
        const std::string pidx = perm ? "op2g_perm" + std::to_string(m) + "[i]" : "i";
        // Index into the offset arrays of `src`: the permutation applies to the
        // offsets as well (pyop2/codegen/builder.py:160-166).
        std::string oidx = pidx;
        if (mi.kind == OP2G_MAP_COMPOSED) {
            const MapInfo &om = S.maps[mi.composed[0]];
            oidx = om.kind == OP2G_MAP_PERMUTED ? "op2g_perm" + std::to_string(mi.composed[0]) + "[i]"
                                                 : "i";
        }
        const bool extr = S.loop.extruded && !sm.offset.empty();
        for (int f = 0; f < nf; ++f) {
            o << ind << "int " << idx_arr(m, f) << "[" << mi.arity << "];\n";
            o << ind << "#pragma unroll\n";
            o << ind << "for (int i = 0; i < " << mi.arity << "; ++i) {\n";
            o << ind << "  int b_ = " << rowname << "[" << (mi.kind == OP2G_MAP_COMPOSED ? "i" : pidx)
              << "];\n";
            if (extr) {
                // pyop2/codegen/builder.py:81-125: base + offset * (layer - bottom + f),
                // with the periodic remainder of :27-30 / :109-121.
                std::string offi = "op2g_off" + std::to_string(src) + "[" + oidx + "]";
                std::string e = "(layer - bottom + " + std::to_string(f) + ")";
                if (S.loop.extruded_periodic) {
                    if (!sm.offset_quotient.empty()) {
                        std::string q = "op2g_offq" + std::to_string(src) + "[" + oidx + "]";
                        e = "(op2g::rem(" + e + " + " + q + ", nlay) - op2g::rem(" + q + ", nlay))";
                    } else {
                        e = "op2g::rem(" + e + ", nlay)";
                    }
                }
                o << ind << "  if (b_ >= 0) b_ += " << offi << " * " << e << ";\n";
            }
            if (S.loop.debug_checks) {
                o << ind << "  if (b_ >= p.toset[" << m
                  << "]) { op2g::set_err(p.err, OP2G_DEVERR_MAP_BOUNDS); b_ = -1; }\n";
            }
            o << ind << "  " << idx_arr(m, f) << "[i] = b_;\n";
            o << ind << "}\n";
        }
    }

    // Staged row of plain map m at entity n: the entries' slots lv<m> from
    // the plan's loc_map (16-bit, read as vectors when the arity allows) and
    // the global targets mv<m> through the partition's slot -> target table
    // and target list in shared memory.
    void emit_staged_row(int m, const std::string &ind) {
        const int ar = S.maps[m].arity;
        const std::string lv = "lv" + std::to_string(m), mv = base_row(m);
        o << ind << "unsigned short " << lv << "[" << ar << "];\n";
        o << ind << "int " << mv << "[" << ar << "];\n";
        o << ind << "{ const unsigned short *r_ = lc" << m << "[mb_] + (n - pbase_) * " << ar << ";\n";
        if (ar % 4 == 0) {
            for (int q = 0; q < ar / 4; ++q)
                o << ind << "  { const ushort4 v_ = ((const ushort4 *)r_)[" << q << "]; " << lv
                  << "[" << 4 * q << "] = v_.x; " << lv << "[" << 4 * q + 1 << "] = v_.y; " << lv
                  << "[" << 4 * q + 2 << "] = v_.z; " << lv << "[" << 4 * q + 3 << "] = v_.w; }\n";
        } else if (ar % 2 == 0) {
            for (int q = 0; q < ar / 2; ++q)
                o << ind << "  { const ushort2 v_ = ((const ushort2 *)r_)[" << q << "]; " << lv
                  << "[" << 2 * q << "] = v_.x; " << lv << "[" << 2 * q + 1 << "] = v_.y; }\n";
        } else {
            o << ind << "#pragma unroll\n";
            o << ind << "  for (int i = 0; i < " << ar << "; ++i) " << lv << "[i] = r_[i];\n";
        }
        o << ind << "#pragma unroll\n";
        o << ind << "  for (int i = 0; i < " << ar << "; ++i) " << mv << "[i] = " << lv
          << "[i] == 0xFFFF ? -1 : si" << m << "[mb_][tg" << m << "[" << lv << "[i]]];\n";
        o << ind << "}\n";
    }

    // Slot of entry `i` of staged argument a's map (the plain map's own
    // entry, or the permuted one); 0xFFFF for a negative entry.
    std::string local_index(size_t a, const std::string &i) const {
        const int m = S.args[a].d.map;
        const int r = st_arg[a];
        if (m == r) return "(int)lv" + std::to_string(r) + "[" + i + "]";
        return "(int)lv" + std::to_string(r) + "[op2g_perm" + std::to_string(m) + "[" + i + "]]";
    }

    // The staged run function.  CTAs take mini-partitions of the plan in turn
    // and pipeline them: the plan segments of partition q + 2 (target list,
    // run offsets, the partition's slots) arrive by bulk copy (one thread
    // issues them; they complete on one of three mbarriers) and the staged
    // READ values and fetched direct arguments of partition q + 1 by
    // per-element asynchronous copies, while partition q computes.  Per
    // partition: a slot -> target table is filled, the iterations run with
    // READ packs from shared memory and INC contributions stored at their
    // slots, then each target's run of slots is summed in slot order and
    // added to the target with one global atomic.  Every mbarrier wait is
    // bounded; when one gives up, the CTA sets OP2G_DEVERR_TIMEOUT in the
    // error word (when there is one), waits (bounded) for its copies in
    // flight and stops.
    void emit_staged_run() {
        std::ostringstream &O = o;
        const int BS = S.block_size;
        staging = true;
        std::vector<int> ms;   // staged maps
        for (size_t m = 0; m < S.maps.size(); ++m)
            if (st_map[m]) ms.push_back((int)m);
        const int NSM = (int)ms.size();
        // the slot -> target table of a staged map is filled only when an
        // argument other than a staged INC goes through it (a staged READ
        // needs its targets' values, any other argument the global targets)
        std::vector<bool> need_tg(S.maps.size(), false);
        for (size_t a = 0; a < S.args.size(); ++a) {
            const op2g_arg_desc &d = S.args[a].d;
            if (d.kind == OP2G_ARG_DAT && st_arg[a] >= 0 && d.access == OP2G_INC) continue;
            auto mark = [&](int m) {
                if (m < 0) return;
                const int r = S.maps[m].kind == OP2G_MAP_PERMUTED ? S.maps[m].base : m;
                if (st_map[r]) need_tg[r] = true;
            };
            if (d.kind == OP2G_ARG_DAT) mark(d.map);
            if (d.kind == OP2G_ARG_MAT) {
                mark(d.map);
                mark(d.cmap);
            }
        }
        for (size_t m = 0; m < S.maps.size(); ++m)
            if (S.maps[m].kind == OP2G_MAP_COMPOSED)
                for (int k = 0; k < S.maps[m].ncomposed; ++k) {
                    const int c = S.maps[m].composed[k];
                    const int r = S.maps[c].kind == OP2G_MAP_PERMUTED ? S.maps[c].base : c;
                    if (st_map[r]) need_tg[r] = true;
                }
        O << "__device__ __forceinline__ void op2g_run_staged(const op2g_params_t &p) {\n";
        O << "  extern __shared__ __align__(16) unsigned char op2g_smem[];\n";
        O << "  __shared__ __align__(8) unsigned long long bar_[3];\n";
        O << "  __shared__ int snu_[3][" << NSM << "];\n";
        emit_global_init();
        // layout (mirrored by staged_smem_bytes on the host)
        O << "  size_t so_ = 0;\n";
        for (int m : ms) {
            const int ar = S.maps[m].arity;
            O << "  const int seg" << m << "_ = (int)((p.smax[" << m << "] + 1 + 7) / 8 * 8);\n";
            O << "  int *si" << m << "[3]; unsigned short *ro" << m << "[3], *lc" << m << "[3];\n";
            O << "  for (int b_ = 0; b_ < 3; ++b_) {\n";
            O << "    si" << m << "[b_] = (int *)(op2g_smem + so_); so_ += ((size_t)seg" << m
              << "_ * 4 + 15) & ~(size_t)15;\n";
            O << "    ro" << m << "[b_] = (unsigned short *)(op2g_smem + so_); so_ += ((size_t)seg" << m
              << "_ * 2 + 15) & ~(size_t)15;\n";
            O << "    lc" << m << "[b_] = (unsigned short *)(op2g_smem + so_); so_ += ((size_t)p.sblock * "
              << ar << " * 2 + 15) & ~(size_t)15;\n";
            O << "  }\n";
            O << "  unsigned short *tg" << m << " = (unsigned short *)(op2g_smem + so_); so_ += "
              << "((size_t)p.sblock * " << ar << " * 2 + 15) & ~(size_t)15;\n";
        }
        for (size_t a = 0; a < S.args.size(); ++a) {
            const op2g_arg_desc &d = S.args[a].d;
            const char *T = ctype_of(d.dtype);
            if (st_arg[a] >= 0 && d.access == OP2G_READ) {
                O << "  " << T << " *sv" << a << "[2];\n";
                O << "  for (int b_ = 0; b_ < 2; ++b_) { sv" << a << "[b_] = (" << T
                  << " *)(op2g_smem + so_); so_ += ((size_t)p.smax[" << st_arg[a] << "] * " << d.dim
                  << " * sizeof(" << T << ") + 15) & ~(size_t)15; }\n";
            } else if (st_arg[a] >= 0) {
                O << "  " << T << " *sv" << a << " = (" << T << " *)(op2g_smem + so_); so_ += ((size_t)p.sblock * "
                  << S.maps[st_arg[a]].arity << " * " << d.dim << " * sizeof(" << T
                  << ") + 15) & ~(size_t)15;\n";
            } else if (st_dir[a]) {
                O << "  " << T << " *dv" << a << "[2];\n";
                O << "  for (int b_ = 0; b_ < 2; ++b_) { dv" << a << "[b_] = (" << T
                  << " *)(op2g_smem + so_); so_ += ((size_t)p.sblock * " << d.dim << " * sizeof(" << T
                  << ") + 15) & ~(size_t)15; }\n";
            }
        }
        O << "  (void)so_;\n";
        O << "  const long long pb1_ = (p.end + p.sblock - 1) / p.sblock;\n";
        O << "  const long long first_ = p.start / p.sblock + blockIdx.x, step_ = gridDim.x;\n";
        O << "  if (threadIdx.x == 0) {\n";
        O << "    for (int b_ = 0; b_ < 3; ++b_) op2g::mbar_init(&bar_[b_], 1);\n";
        O << "    op2g::fence_mbar_init();\n";
        O << "  }\n";
        O << "  __syncthreads();\n";
        O << "  unsigned ph_[3] = {0u, 0u, 0u};   // parity of each plan buffer's next phase\n";
        O << "  bool pend_[3] = {false, false, false};   // a bulk copy into the buffer is in flight\n";
        // thread 0 holds the plan offsets of the next partition to issue
        O << "  long long po_[" << NSM << "], pl_[" << NSM << "]; int pn_[" << NSM << "];\n";
        O << "  auto load_next_ = [&](long long q_) {\n";
        O << "    if (threadIdx.x != 0 || q_ >= pb1_) return;\n";
        for (int i = 0; i < NSM; ++i) {
            const int m = ms[i];
            O << "    po_[" << i << "] = p.soff[" << m << "][q_]; pl_[" << i << "] = p.soff[" << m
              << "][q_ + 1] - po_[" << i << "]; pn_[" << i << "] = p.snum[" << m << "][q_];\n";
        }
        O << "  };\n";
        // the plan segments of partition q into plan buffer b (thread 0 issues)
        O << "  auto issue_meta_ = [&](long long q_, int b_) {\n";
        O << "    if (q_ >= pb1_) return;\n";
        O << "    pend_[b_] = true;\n";
        O << "    if (threadIdx.x != 0) return;\n";
        O << "    const long long qb_ = q_ * p.sblock;\n";
        O << "    const long long qe_ = qb_ + p.sblock < p.end ? qb_ + p.sblock : p.end;\n";
        O << "    unsigned bytes_ = 0;\n";
        for (int i = 0; i < NSM; ++i) {
            const int m = ms[i], ar = S.maps[m].arity;
            O << "    const unsigned lb" << i << "_ = (unsigned)(((qe_ - qb_) * " << ar
              << " * 2 + 15) & ~15LL);\n";
            O << "    bytes_ += (unsigned)pl_[" << i << "] * 6u + lb" << i << "_;\n";
            O << "    snu_[b_][" << i << "] = pn_[" << i << "];\n";
        }
        O << "    op2g::mbar_expect_tx(&bar_[b_], bytes_);\n";
        for (int i = 0; i < NSM; ++i) {
            const int m = ms[i], ar = S.maps[m].arity;
            O << "    op2g::bulk_g2s(si" << m << "[b_], p.sind[" << m << "] + po_[" << i
              << "], (unsigned)pl_[" << i << "] * 4u, &bar_[b_]);\n";
            O << "    op2g::bulk_g2s(ro" << m << "[b_], p.sruns[" << m << "] + po_[" << i
              << "], (unsigned)pl_[" << i << "] * 2u, &bar_[b_]);\n";
            O << "    op2g::bulk_g2s(lc" << m << "[b_], p.sloc[" << m << "] + qb_ * " << ar << ", lb"
              << i << "_, &bar_[b_]);\n";
        }
        O << "    load_next_(q_ + step_);\n";
        O << "  };\n";
        // the value copies of partition q (plan buffer mb, value buffer vb)
        O << "  auto issue_vals_ = [&](long long q_, int qm_, int qv_) {\n";
        O << "    if (q_ >= pb1_) return;\n";
        O << "    const long long q0_ = q_ * p.sblock > p.start ? q_ * p.sblock : p.start;\n";
        O << "    const long long q1_ = (q_ + 1) * p.sblock < p.end ? (q_ + 1) * p.sblock : p.end;\n";
        O << "    (void)q0_; (void)q1_; (void)qm_; (void)qv_;\n";
        for (size_t a = 0; a < S.args.size(); ++a) {
            const op2g_arg_desc &d = S.args[a].d;
            const char *T = ctype_of(d.dtype);
            const size_t e = elt_size(d.dtype);
            if (st_arg[a] >= 0 && d.access == OP2G_READ) {
                const int r = st_arg[a];
                int qi = 0;
                while (ms[qi] != r) ++qi;
                O << "    for (int k_ = threadIdx.x; k_ < snu_[qm_][" << qi << "] * " << d.dim << "; k_ += "
                  << BS << ") {\n";
                O << "      const int v_ = k_ / " << d.dim << ";\n";
                O << "      op2g::cp_async<" << e << ">(sv" << a << "[qv_] + k_, (const " << T
                  << " *)p.ptr[" << S.args[a].slot << "] + (long long)si" << r << "[qm_][v_] * "
                  << gstride(a) << " + (k_ - v_ * " << d.dim << "));\n";
                O << "    }\n";
            } else if (st_arg[a] < 0 && st_dir[a]) {
                O << "    for (int k_ = threadIdx.x; k_ < (int)(q1_ - q0_) * " << d.dim << "; k_ += " << BS
                  << ") {\n";
                O << "      const int v_ = k_ / " << d.dim << ";\n";
                O << "      op2g::cp_async<" << e << ">(dv" << a << "[qv_] + k_, (const " << T << " *)p.ptr["
                  << S.args[a].slot << "] + (q0_ + v_) * " << gstride(a) << " + (k_ - v_ * " << d.dim
                  << "));\n";
                O << "    }\n";
            }
        }
        O << "  };\n";
        O << "  bool ok_ = true;\n";
        // prologue: plan segments of the first two partitions, values of the first
        O << "  load_next_(first_);\n";
        O << "  issue_meta_(first_, 0);\n";
        O << "  issue_meta_(first_ + step_, 1);\n";
        O << "  if (first_ < pb1_) {\n";
        O << "    ok_ = op2g::mbar_wait(&bar_[0], ph_[0]);\n";
        O << "    if (ok_) { ph_[0] ^= 1u; pend_[0] = false; }\n";
        O << "    ok_ = __syncthreads_and(ok_);\n";
        O << "    if (ok_) issue_vals_(first_, 0, 0);\n";
        O << "  }\n";
        O << "  op2g::cp_async_commit();\n";
        O << "  int mb_ = 0, vb_ = 0;\n";
        O << "  for (long long pb_ = first_; ok_ && pb_ < pb1_; pb_ += step_) {\n";
        O << "    const int mbn_ = mb_ == 2 ? 0 : mb_ + 1, mbn2_ = mbn_ == 2 ? 0 : mbn_ + 1;\n";
        O << "    if (pb_ + step_ < pb1_) {\n";
        O << "      ok_ = op2g::mbar_wait(&bar_[mbn_], ph_[mbn_]);\n";
        O << "      if (ok_) { ph_[mbn_] ^= 1u; pend_[mbn_] = false; }\n";
        O << "      if (!__syncthreads_and(ok_)) { ok_ = false; break; }\n";
        O << "      issue_vals_(pb_ + step_, mbn_, vb_ ^ 1);\n";
        O << "    }\n";
        O << "    op2g::cp_async_commit();\n";
        O << "    op2g::cp_async_wait<1>();   // this partition's values\n";
        O << "    __syncthreads();\n";
        // buffer mbn2_ was last read by the previous partition, whose final
        // barrier (with the proxy fence before it) ordered those reads
        O << "    issue_meta_(pb_ + 2 * step_, mbn2_);\n";
        O << "    const long long pbase_ = pb_ * p.sblock;\n";
        O << "    const long long c0_ = pbase_ > p.start ? pbase_ : p.start;\n";
        O << "    const long long c1_ = pbase_ + p.sblock < p.end ? pbase_ + p.sblock : p.end;\n";
        bool fill = false;
        for (int i = 0; i < NSM; ++i) {
            const int m = ms[i];
            O << "    const int nu" << m << "_ = snu_[mb_][" << i << "];\n";
            if (!need_tg[m]) continue;
            fill = true;
            O << "    for (int k_ = threadIdx.x; k_ < nu" << m << "_; k_ += " << BS << ")\n";
            O << "      for (int s_ = ro" << m << "[mb_][k_]; s_ < ro" << m << "[mb_][k_ + 1]; ++s_) tg" << m
              << "[s_] = (unsigned short)k_;\n";
        }
        bool zero = false;
        for (size_t a = 0; a < S.args.size(); ++a)
            zero = zero || (st_arg[a] >= 0 && S.args[a].d.access == OP2G_INC);
        if (zero) {
            // a partition cut by [start, end) leaves the slots of the entries
            // outside unstored: they must add 0
            O << "    const long long pe_ = pbase_ + p.sblock < p.sn ? pbase_ + p.sblock : p.sn;\n";
            O << "    if (c0_ != pbase_ || c1_ != pe_) {\n";
            for (size_t a = 0; a < S.args.size(); ++a) {
                if (st_arg[a] < 0 || S.args[a].d.access != OP2G_INC) continue;
                const int D = S.args[a].d.dim, r = st_arg[a];
                O << "      for (int k_ = threadIdx.x; k_ < (int)ro" << r << "[mb_][nu" << r << "_] * " << D
                  << "; k_ += " << BS << ") sv" << a << "[k_] = (" << ctype_of(S.args[a].d.dtype)
                  << ")0;\n";
            }
            O << "    }\n";
        }
        if (fill || zero) O << "    __syncthreads();\n";
        O << "    for (long long it = c0_ + threadIdx.x; it < c1_; it += " << BS << ") {\n";
        O << "      const long long n = it;\n";
        emit_body("      ", false, false);
        O << "    }\n";
        O << "    __syncthreads();\n";
        for (size_t a = 0; a < S.args.size(); ++a) {
            if (st_arg[a] < 0 || S.args[a].d.access != OP2G_INC) continue;
            const op2g_arg_desc &d = S.args[a].d;
            const char *T = ctype_of(d.dtype);
            const int D = d.dim, r = st_arg[a];
            O << "    for (int k_ = threadIdx.x; k_ < nu" << r << "_ * " << D << "; k_ += " << BS
              << ") {\n";
            O << "      const int v_ = k_ / " << D << ", j_ = k_ - v_ * " << D << ";\n";
            O << "      " << T << " s_ = (" << T << ")0;\n";
            O << "      for (int q_ = ro" << r << "[mb_][v_]; q_ < ro" << r << "[mb_][v_ + 1]; ++q_) s_ += sv" << a
              << "[q_ * " << D << " + j_];\n";
            O << "      op2g::atomic_inc((" << T << " *)p.ptr[" << S.args[a].slot << "] + (long long)si"
              << r << "[mb_][v_] * " << gstride(a) << " + j_, s_);\n";
            O << "    }\n";
        }
        // this partition's plan buffer is refilled by bulk copy two partitions on
        O << "    op2g::fence_proxy_async_smem();\n";
        O << "    __syncthreads();\n";
        O << "    mb_ = mbn_;\n";
        O << "    vb_ ^= 1;\n";
        O << "  }\n";
        O << "  op2g::cp_async_wait<0>();\n";
        O << "  if (!ok_) {\n";
        O << "    if (threadIdx.x == 0) op2g::set_err(p.err, OP2G_DEVERR_TIMEOUT);\n";
        O << "    for (int b_ = 0; b_ < 3; ++b_)\n";
        O << "      if (pend_[b_]) (void)op2g::mbar_wait(&bar_[b_], ph_[b_]);\n";
        O << "    __syncthreads();\n";
        O << "    return;\n";
        O << "  }\n";
        emit_global_reductions();
        O << "}\n\n";
        staging = false;
    }

    // Per-thread accumulators of Global INC/MIN/MAX arguments.
    void emit_global_init() {
        std::ostringstream &O = o;
        for (size_t a = 0; a < S.args.size(); ++a) {
            const ArgInfo &A = S.args[a];
            if (A.d.kind != OP2G_ARG_GLOBAL) continue;
            const char *T = ctype_of(A.d.dtype);
            if (A.d.access == OP2G_INC) {
                O << "  " << T << " gacc" << a << "[" << A.d.dim << "];\n";
                O << "  for (int j = 0; j < " << A.d.dim << "; ++j) gacc" << a << "[j] = (" << T
                  << ")0;\n";
            } else if (A.d.access == OP2G_MIN || A.d.access == OP2G_MAX) {
                O << "  " << T << " gacc" << a << "[" << A.d.dim << "];\n";
                O << "  for (int j = 0; j < " << A.d.dim << "; ++j) gacc" << a << "[j] = ((const "
                  << T << " *)p.ptr[" << A.slot << "])[j];\n";
            }
        }
    }

    // Warp-reduced Global results, one atomic per warp (pyop2/parloop.py:
    // 409-452 semantics on one device: INC goes to the zeroed temporary,
    // MIN/MAX straight into the Global).
    void emit_global_reductions() {
        std::ostringstream &O = o;
        for (size_t a = 0; a < S.args.size(); ++a) {
            const ArgInfo &A = S.args[a];
            if (A.d.kind != OP2G_ARG_GLOBAL || A.d.access == OP2G_READ) continue;
            const char *T = ctype_of(A.d.dtype);
            const char *red = A.d.access == OP2G_INC ? "warp_sum"
                              : A.d.access == OP2G_MIN ? "warp_min" : "warp_max";
            const char *atom = A.d.access == OP2G_INC ? "atomic_inc"
                               : A.d.access == OP2G_MIN ? "atomic_min" : "atomic_max";
            O << "  for (int j = 0; j < " << A.d.dim << "; ++j) {\n";
            O << "    " << T << " v_ = op2g::" << red << "(gacc" << a << "[j]);\n";
            O << "    if ((threadIdx.x & 31) == 0) op2g::" << atom << "(((" << T << " *)p.ptr["
              << A.slot << "]) + j, v_);\n";
            O << "  }\n";
        }
    }

    std::string emit() {
        std::ostringstream &O = o;
        O << "// generated by op2g_codegen.cpp for kernel '" << S.kernel_name << "'\n";
        O << "#include \"op2g_device.cuh\"\n";
        O << "#define OP2G_DEVERR_MAP_BOUNDS " << OP2G_DEVERR_MAP_BOUNDS << "\n";
        O << "#define OP2G_DEVERR_NEW_NONZERO " << OP2G_DEVERR_NEW_NONZERO << "\n";
        O << "#define OP2G_DEVERR_TIMEOUT " << OP2G_DEVERR_TIMEOUT << "\n";
        O << "namespace op2g { __device__ __forceinline__ int rem(int a, int b) { return a < b ? a : a - b; } }\n";
        O << "#define restrict __restrict__\n";
        O << "// ---- user kernel ----\n";
        O << strip_system_includes(S.user_src) << "\n";
        O << "// ---- end of user kernel ----\n";
        O << "#undef restrict\n";
        emit_constants();
        const int nptr = S.nptrs;
        const int nmaps = (int)S.maps.size();
        O << "struct op2g_params_t {\n"
          << "  long long start, end;\n"
          << "  const int *layers;\n"
          << "  const int *indices;\n"
          << "  int *err;\n"
          << "  void *ptr[" << (nptr > 0 ? nptr : 1) << "];\n"
          << "  long long toset[" << (nmaps > 0 ? nmaps : 1) << "];\n";
        if (any_staged) {
            // the staging plan (op2g_stage_desc), one entry per map
            const int nm = nmaps > 0 ? nmaps : 1;
            O << "  long long sblock, sn;\n"
              << "  long long smax[" << nm << "];\n"
              << "  const int *sind[" << nm << "];\n"
              << "  const long long *soff[" << nm << "];\n"
              << "  const int *snum[" << nm << "];\n"
              << "  const unsigned short *sruns[" << nm << "];\n"
              << "  const unsigned short *sloc[" << nm << "];\n";
        }
        O << "};\n";

        const int BS = S.block_size;
        bool warp = S.loop.scatter == OP2G_SCATTER_WARP;
        const bool plain = S.loop.scatter == OP2G_SCATTER_PLAIN;
        const bool extr = S.loop.extruded != 0;
        // One thread per column (layers in sequence) when layers differ per
        // column, when a colour's launch must not touch a column twice in
        // parallel, or when a direct argument is written: direct arguments are
        // indexed by the column only (pyop2/codegen/builder.py:367-377), so the
        // layers of one column update the same entry and must run in order.
        bool direct_written = false;
        for (const ArgInfo &A : S.args)
            if (A.d.kind == OP2G_ARG_DAT && A.d.map < 0 && A.d.access != OP2G_READ)
                direct_written = true;
        const bool varlay = extr && (!S.loop.constant_layers || plain || direct_written);
        if (varlay) warp = false;  // lanes of a warp run different layer counts
        if (has_groups) warp = false;  // grouped packs scatter by atomics
        plan_shared(!extr && S.loop.scatter == OP2G_SCATTER_SHARED);

        // ----- the run function: a strided sweep of [start, end) plus reductions
        O << "__device__ __forceinline__ void op2g_run(const op2g_params_t &p, long long start, "
             "long long end, long long first, long long stride) {\n";
        emit_global_init();
        if (extr) {
            // pyop2/codegen/builder.py:771-812 (layer extents per iteration region)
            O << "  const int *lay_ = p.layers;\n";
        }
        std::string ent_expr = "n";
        if (extr && !varlay) {
            O << "  const int cs_ = lay_[0], ce_ = lay_[1] - 1;  // cellStart, cellEnd\n";
            emit_layer_extents("cs_", "ce_", "ls_", "le_", "  ");
            O << "  const long long nl_ = le_ > ls_ ? (long long)(le_ - ls_) : 0;\n";
            O << "  const long long i0_ = start * nl_, i1_ = end * nl_;\n";
        } else {
            O << "  const long long i0_ = start, i1_ = end;\n";
        }
        // Prefetch (non-extruded loops): the map rows of a thread's next
        // iteration are loaded before its current iteration runs.
        const bool pf = S.loop.prefetch && !extr;
        const std::vector<bool> rows = row_maps();
        auto ent_of = [&](const std::string &itx) {
            return S.loop.indexed ? "(long long)p.indices[" + itx + "]" : itx;
        };
        if (pf) {
            O << "  const long long pit0_ = i0_ + first + threadIdx.x;\n";
            for (size_t m = 0; m < S.maps.size(); ++m)
                if (rows[m])
                    O << "  int pf" << m << "[" << S.maps[m].arity << "] = {0};\n";
            O << "  if (pit0_ < i1_) {\n    const long long pn_ = " << ent_of("pit0_") << ";\n";
            for (size_t m = 0; m < S.maps.size(); ++m)
                if (rows[m]) emit_plain_row((int)m, "pn_", "    ", "pf" + std::to_string(m), false);
            O << "  }\n";
        }
        for (size_t a = 0; a < S.args.size(); ++a)
            if (shared_ts[a]) {
                // keys, sums, the list of claimed slots and its length (two
                // counters used by alternate sweep steps)
                O << "  __shared__ int sk" << a << "[" << shared_ts[a] << "];\n";
                O << "  __shared__ " << ctype_of(S.args[a].d.dtype) << " sv" << a << "["
                  << shared_ts[a] * S.args[a].d.dim << "];\n";
                O << "  __shared__ int sl" << a << "[" << shared_ts[a] << "];\n";
                O << "  __shared__ int sn" << a << "[2];\n";
            }
        if (any_shared) O << "  int par_ = 0;\n";
        if (any_shared) {
            // tables start empty; each sweep step's flush empties them again
            for (size_t a = 0; a < S.args.size(); ++a)
                if (shared_ts[a]) {
                    const int D = S.args[a].d.dim;
                    O << "  for (int s_ = threadIdx.x; s_ < " << shared_ts[a] << "; s_ += " << BS
                      << ") { sk" << a << "[s_] = -1;";
                    O << " for (int j = 0; j < " << D << "; ++j) sv" << a << "[s_ * " << D
                      << " + j] = (" << ctype_of(S.args[a].d.dtype) << ")0; }\n";
                    O << "  if (threadIdx.x == 0) { sn" << a << "[0] = 0; sn" << a << "[1] = 0; }\n";
                }
            O << "  __syncthreads();\n";
        }
        // Cells per thread: loops without direct RW/INC/MIN/MAX arguments (a
        // clamped iteration reruns the last one, which for a direct WRITE
        // argument stores the same values again, but would apply an update
        // twice), passthrough arguments, warp or shared-memory scatter or
        // map-row prefetch.
        bool has_pass = false, direct_update = false;
        for (const ArgInfo &A : S.args) {
            has_pass = has_pass || A.d.kind == OP2G_ARG_PASSTHROUGH;
            direct_update = direct_update || (A.d.kind == OP2G_ARG_DAT && A.d.map < 0 &&
                                              A.d.access != OP2G_READ && A.d.access != OP2G_WRITE);
        }
        const int cpt = (S.loop.cells_per_thread > 1 && !warp && !any_shared && !pf && !varlay &&
                         !direct_update && !has_pass)
                            ? S.loop.cells_per_thread
                            : 1;
        cells_per_thread = cpt;
        if (cpt > 1) {
            guard_unpack = true;
            O << "  for (long long base_ = i0_ + first; base_ < i1_; base_ += stride * " << cpt << ") {\n";
            O << "#pragma unroll\n";
            O << "   for (int c_ = 0; c_ < " << cpt << "; ++c_) {\n";
            O << "    const long long ic_ = base_ + c_ * stride + threadIdx.x;\n";
            O << "    const bool active = ic_ < i1_;\n";
            O << "    const long long it = active ? ic_ : i1_ - 1;\n";
        } else {
            O << "  for (long long base_ = i0_ + first; base_ < i1_; base_ += stride) {\n";
            O << "    const long long it = base_ + threadIdx.x;\n";
            O << "    const bool active = it < i1_;\n";
        }
        if (pf) {
            for (size_t m = 0; m < S.maps.size(); ++m)
                if (rows[m])
                    O << "    int nx" << m << "[" << S.maps[m].arity << "] = {0};\n";
            O << "    if (it + stride < i1_) {\n      const long long pn_ = "
              << ent_of("(it + stride)") << ";\n";
            for (size_t m = 0; m < S.maps.size(); ++m)
                if (rows[m]) emit_plain_row((int)m, "pn_", "      ", "nx" + std::to_string(m), false);
            O << "    }\n";
        }
        // Pack declarations visible to the warp-aggregated unpack.
        std::string I = "    ";
        // Per-iteration declarations that warp scatter needs outside `if (active)`.
        if (warp) {
            for (size_t a = 0; a < S.args.size(); ++a) {
                const ArgInfo &A = S.args[a];
                if (A.d.kind == OP2G_ARG_DAT && A.d.map >= 0 && A.d.access == OP2G_INC) {
                    const int ar = S.maps[A.d.map].arity;
                    O << I << ctype_of(A.d.dtype) << " t" << a << "[" << nf * ar * A.d.dim
                      << "];\n";
                    O << I << "int ti" << a << "[" << nf * ar << "];\n";
                }
            }
        }
        O << I << (cpt > 1 ? "{\n" : "if (active) {\n");
        std::string J = "      ";
        // entity / layer
        if (extr && !varlay) {
            O << J << "const long long it_ent = it / nl_;\n";
            O << J << "const int layer = ls_ + (int)(it - it_ent * nl_);\n";
            O << J << "const long long n = " << (S.loop.indexed ? "p.indices[it_ent]" : "it_ent")
              << ";\n";
            O << J << "const int bottom = " << (S.loop.iteration_region == OP2G_ON_TOP ? "cs_" : "ls_")
              << ";\n";
            O << J << "const int nlay = ce_ - cs_; (void)nlay; (void)bottom;\n";
            emit_body(J, warp, plain);
        } else if (varlay) {
            O << J << "const long long n = " << (S.loop.indexed ? "p.indices[it]" : "it") << ";\n";
            if (S.loop.constant_layers)
                O << J << "const int cs_ = lay_[0], ce_ = lay_[1] - 1;\n";
            else
                O << J << "const int cs_ = lay_[2 * n], ce_ = lay_[2 * n + 1] - 1;\n";
            emit_layer_extents("cs_", "ce_", "ls_", "le_", J);
            O << J << "const int bottom = " << (S.loop.iteration_region == OP2G_ON_TOP ? "cs_" : "ls_")
              << ";\n";
            O << J << "const int nlay = ce_ - cs_; (void)nlay; (void)bottom;\n";
            O << J << "for (int layer = ls_; layer < le_; ++layer) {\n";
            emit_body(J + "  ", false, plain);
            O << J << "}\n";
        } else {
            O << J << "const long long n = " << (S.loop.indexed ? "p.indices[it]" : "it") << ";\n";
            // The next sweep step's rows of direct arguments that are read
            // are prefetched into L2: the kernel's loads through them cannot
            // move above its stores through other Dat pointers (the compiler
            // cannot prove them distinct), so each thread would otherwise
            // keep one load in flight (a 12.58 M-cell direct copy: 0.042 ->
            // 0.037 ms; a prefetch is a hint, nothing it reads is used).
            if (!S.loop.indexed && cpt == 1 && !staging) {
                bool any = false;
                for (size_t a = 0; a < S.args.size(); ++a) {
                    const op2g_arg_desc &d = S.args[a].d;
                    if (d.kind != OP2G_ARG_DAT || d.map >= 0 || d.access == OP2G_WRITE) continue;
                    if (!any) O << J << "if (it + stride < i1_) {\n";
                    any = true;
                    O << J << "  asm volatile(\"prefetch.global.L2 [%0];\" :: \"l\"(("
                      << ctype_of(d.dtype) << " *)p.ptr[" << S.args[a].slot << "] + (it + stride) * "
                      << gstride(a) << "));\n";
                }
                if (any) O << J << "}\n";
            }
            emit_body(J, warp, plain, pf);
        }
        O << I << "}\n";
        if (pf) {
            for (size_t m = 0; m < S.maps.size(); ++m)
                if (rows[m])
                    O << I << "#pragma unroll\n" << I << "for (int i = 0; i < " << S.maps[m].arity
                      << "; ++i) pf" << m << "[i] = nx" << m << "[i];\n";
        }
        if (warp) {
            for (size_t a = 0; a < S.args.size(); ++a) {
                const ArgInfo &A = S.args[a];
                if (A.d.kind == OP2G_ARG_DAT && A.d.map >= 0 && A.d.access == OP2G_INC) {
                    const int ar = S.maps[A.d.map].arity;
                    const int D = A.d.dim;
                    const char *T = ctype_of(A.d.dtype);
                    O << I << "{ " << T << " *d_ = (" << T << " *)p.ptr[" << A.slot << "];\n";
                    O << I << "#pragma unroll\n";
                    O << I << "  for (int i = 0; i < " << nf * ar << "; ++i) {\n";
                    O << I << "    const bool v_ = active && ti" << a << "[i] >= 0;\n";
                    O << I << "    const long long o_ = v_ ? (long long)ti" << a << "[i] * "
                      << gstride(a) << " : 0;\n";
                    O << I << "#pragma unroll\n";
                    O << I << "    for (int j = 0; j < " << D << "; ++j) op2g::warp_agg_inc(d_ + o_ + j, t"
                      << a << "[i * " << D << " + j], v_);\n";
                    O << I << "  } }\n";
                }
            }
        }
        if (any_shared) {
            // The sweep step is uniform across the CTA (base_ depends on the
            // block only), so these barriers are reached by every thread.
            O << "    __syncthreads();\n";
            for (size_t a = 0; a < S.args.size(); ++a)
                if (shared_ts[a]) {
                    const int D = S.args[a].d.dim;
                    const char *T = ctype_of(S.args[a].d.dtype);
                    O << "    { " << T << " *d_ = (" << T << " *)p.ptr[" << S.args[a].slot << "];\n";
                    O << "      const int n_ = sn" << a << "[par_];\n";
                    O << "      if (threadIdx.x == 0) sn" << a << "[par_ ^ 1] = 0;\n";
                    O << "      for (int s_ = threadIdx.x; s_ < n_; s_ += " << BS
                      << ") { const int h_ = sl" << a << "[s_]; const int k_ = sk" << a
                      << "[h_]; sk" << a << "[h_] = -1;\n";
                    O << "        for (int j = 0; j < " << D << "; ++j) { op2g::atomic_inc(&d_[(long long)k_ * "
                      << gstride(a) << " + j], sv" << a << "[h_ * " << D << " + j]); sv" << a << "[h_ * " << D
                      << " + j] = (" << T << ")0; } } }\n";
                }
            O << "    __syncthreads();\n";
            O << "    par_ ^= 1;\n";
        }
        if (cpt > 1) O << "   }\n";  // cells of the step
        O << "  }\n";  // sweep loop
        guard_unpack = false;
        emit_global_reductions();
        O << "}\n\n";

        // ----- the entry points.  Without shared-memory staging (whose
        // tables are sized for BS threads) the wrapper may be launched with
        // fewer threads per CTA than BS: a small iteration set is then
        // spread over more SMs (each SM issues FP64 at 2 per clock).
        const std::string bdim = any_shared ? std::to_string(BS) : std::string("blockDim.x");
        if (any_staged) {
            emit_staged_run();
            O << "extern \"C\" __global__ void __launch_bounds__(" << BS
              << ") op2g_wrap(const __grid_constant__ op2g_params_t p) {\n"
              << "  op2g_run_staged(p);\n}\n";
        } else {
            O << "extern \"C\" __global__ void __launch_bounds__(" << BS
              << ") op2g_wrap(const __grid_constant__ op2g_params_t p) {\n"
              << "  op2g_run(p, p.start, p.end, (long long)blockIdx.x * " << bdim
              << ", (long long)gridDim.x * " << bdim << ");\n}\n";
        }
        if (!any_shared && !any_staged) {
            // Balanced form for launches of a few CTAs per SM: CTA b takes the
            // b-th of gridDim.x equal contiguous chunks of the entities, so a
            // grid of k CTAs per SM gives every SM the same work.
            O << "extern \"C\" __global__ void __launch_bounds__(" << BS
              << ") op2g_wrap_chunked(const __grid_constant__ op2g_params_t p) {\n"
              << "  const long long n_ = p.end - p.start;\n"
              << "  const long long c_ = (n_ + gridDim.x - 1) / gridDim.x;\n"
              << "  const long long s_ = p.start + (long long)blockIdx.x * c_;\n"
              << "  const long long e_ = s_ + c_ < p.end ? s_ + c_ : p.end;\n"
              << "  if (s_ < e_) op2g_run(p, s_, e_, 0, (long long)blockDim.x);\n}\n";
        }
        O << "extern \"C\" __global__ void __launch_bounds__(" << BS
          << ") op2g_wrap_batched(const op2g_params_t *__restrict__ P, const long long "
             "*__restrict__ work, long long nwork) {\n"
          << "  for (long long w = blockIdx.x; w < nwork; w += gridDim.x) {\n"
          << "    const op2g_params_t &p = P[work[3 * w]];\n"
          << "    op2g_run(p, work[3 * w + 1], work[3 * w + 2], 0, " << BS << ");\n"
          << "  }\n}\n";
        return O.str();
    }

    // Layer range for the iteration region (pyop2/codegen/builder.py:771-800).
    void emit_layer_extents(const std::string &cs, const std::string &ce, const std::string &ls,
                            const std::string &le, const std::string &ind) {
        switch (S.loop.iteration_region) {
            case OP2G_ON_BOTTOM:
                o << ind << "const int " << ls << " = " << cs << ", " << le << " = " << cs << " + 1;\n";
                break;
            case OP2G_ON_TOP:
                o << ind << "const int " << ls << " = " << ce << " - 1, " << le << " = " << ce << ";\n";
                break;
            case OP2G_ON_INTERIOR_FACETS:
                if (S.loop.extruded_periodic)
                    o << ind << "const int " << ls << " = " << cs << ", " << le << " = " << ce << ";\n";
                else
                    o << ind << "const int " << ls << " = " << cs << ", " << le << " = " << ce
                      << " - 1;\n";
                break;
            default:
                o << ind << "const int " << ls << " = " << cs << ", " << le << " = " << ce << ";\n";
        }
    }

    // Pack, call, unpack for one iteration (entity n, and layer when extruded).
    void emit_body(const std::string &J, bool warp, bool plain, bool rows_prefetched = false) {
        std::ostringstream &O = o;
        std::vector<bool> used = used_maps();
        std::vector<bool> need_row = row_maps();
        for (size_t m = 0; m < S.maps.size(); ++m) {
            if (!need_row[m]) continue;
            if (staging && st_map[m]) {
                emit_staged_row((int)m, J);
                continue;
            }
            if (rows_prefetched) {
                O << J << "int " << base_row((int)m) << "[" << S.maps[m].arity << "];\n";
                O << J << "#pragma unroll\n" << J << "for (int i = 0; i < " << S.maps[m].arity
                  << "; ++i) " << base_row((int)m) << "[i] = pf" << m << "[i];\n";
            } else {
                emit_plain_row((int)m, "n", J);
            }
        }
        for (size_t m = 0; m < S.maps.size(); ++m)
            if (used[m]) emit_index_arrays((int)m, J);

        // Packs (pyop2/codegen/builder.py:240-300, 303-365, 531-552)
        std::vector<std::string> kargs;
        for (size_t a = 0; a < S.args.size(); ++a) {
            const ArgInfo &A = S.args[a];
            const char *T = ctype_of(A.d.dtype);
            const std::string an = std::to_string(a);
            if (A.d.kind == OP2G_ARG_PASSTHROUGH) {
                kargs.push_back("op2g::ptr((" + std::string(T) + " *)p.ptr[" +
                                std::to_string(A.slot) + "])");
            } else if (A.d.kind == OP2G_ARG_GLOBAL) {
                if (A.d.access == OP2G_READ) {
                    kargs.push_back("op2g::ptr((" + std::string(T) + " *)p.ptr[" +
                                    std::to_string(A.slot) + "])");
                } else {
                    O << J << T << " g" << an << "[" << A.d.dim << "];\n";
                    if (A.d.access == OP2G_INC)
                        O << J << "for (int j = 0; j < " << A.d.dim << "; ++j) g" << an << "[j] = "
                          << inc_zero(A.d.dtype) << ";\n";
                    else
                        O << J << "for (int j = 0; j < " << A.d.dim << "; ++j) g" << an
                          << "[j] = gacc" << an << "[j];\n";
                    kargs.push_back("op2g::ptr(g" + an + ")");
                }
            } else if (A.d.kind == OP2G_ARG_DAT) {
                const int D = A.d.dim;
                if (A.d.map < 0) {
                    // direct: pointer into the Dat (pyop2/codegen/builder.py:367-377);
                    // in a staged wrapper a fetched READ argument is read from
                    // its partition buffer in shared memory
                    if (staging && st_dir[a])
                        kargs.push_back("op2g::ptr((" + std::string(T) + " *)dv" + an +
                                        "[vb_] + (n - c0_) * " + std::to_string(A.d.dim) + ")");
                    else {
                        // in the variant launched on aligned pointers the
                        // compiler is told each row's alignment, so the
                        // kernel's accesses to adjacent components merge
                        // into vector loads and stores
                        const int al = align_hints ? direct_row_alignment(S, a) : 0;
                        const std::string row = "(" + std::string(T) + " *)p.ptr[" +
                                                std::to_string(A.slot) + "] + n * " +
                                                std::to_string(gstride(a));
                        kargs.push_back(al ? "op2g::ptr((" + std::string(T) +
                                                 " *)__builtin_assume_aligned(" + row + ", " +
                                                 std::to_string(al) + "))"
                                           : "op2g::ptr(" + row + ")");
                    }
                    continue;
                }
                const int ar = S.maps[A.d.map].arity;
                const bool lead = first[a] == (int)a;
                const int tot = psize[first[a]];
                const std::string tn = "t" + std::to_string(first[a]);
                const std::string po = std::to_string(poff[a]) + " + ";
                const bool decl_outside = warp && A.d.access == OP2G_INC;
                if (lead && !decl_outside) O << J << T << " " << tn << "[" << tot << "];\n";
                if (A.d.access == OP2G_INC || A.d.access == OP2G_WRITE) {
                    if (lead) {
                        O << J << "#pragma unroll\n";
                        O << J << "for (int k = 0; k < " << tot << "; ++k) " << tn << "[k] = "
                          << (A.d.access == OP2G_INC ? inc_zero(A.d.dtype)
                                                     : "(" + std::string(T) + ")0")
                          << ";\n";
                    }
                } else if (staging && st_arg[a] >= 0) {
                    // staged: the partition's values sit at the entry's target
                    O << J << "#pragma unroll\n";
                    O << J << "for (int i = 0; i < " << ar << "; ++i) {\n";
                    O << J << "  const int l_ = " << local_index(a, "i") << ";\n";
                    O << J << "  const int q_ = l_ != 0xFFFF ? (int)tg" << st_arg[a] << "[l_] : -1;\n";
                    O << J << "#pragma unroll\n";
                    O << J << "  for (int j = 0; j < " << D << "; ++j) " << tn << "[" << po
                      << "i * " << D << " + j] = q_ >= 0 ? sv" << a << "[vb_][q_ * " << D
                      << " + j] : (" << T << ")0;\n";
                    O << J << "}\n";
                } else {
                    O << J << "{ const " << T << " *d_ = (const " << T << " *)p.ptr[" << A.slot
                      << "];\n";
                    for (int f = 0; f < nf; ++f) {
                        O << J << "#pragma unroll\n";
                        O << J << "  for (int i = 0; i < " << ar << "; ++i) {\n";
                        O << J << "    const int x_ = " << idx_arr(A.d.map, f) << "[i];\n";
                        O << J << "#pragma unroll\n";
                        const bool nc = S.loop.nc_reads && A.d.access == OP2G_READ;
                        O << J << "    for (int j = 0; j < " << D << "; ++j) " << tn << "[" << po
                          << "(" << f * ar << " + i) * " << D << " + j] = x_ >= 0 ? "
                          << (nc ? "__ldg(&" : "") << "d_[(long long)x_ * " << gstride(a) << " + j]"
                          << (nc ? ")" : "") << " : (" << T << ")0;\n";
                        O << J << "  }\n";
                    }
                    O << J << "}\n";
                }
                if (lead) kargs.push_back("op2g::ptr(" + tn + ")");
            } else if (A.d.kind == OP2G_ARG_MAT) {
                if (first[a] != (int)a) continue;   // a later block of a mixed Mat
                const int tot = psize[a];
                O << J << T << " t" << an << "[" << tot << "];\n";
                O << J << "#pragma unroll\n";
                O << J << "for (int k = 0; k < " << tot << "; ++k) t" << an << "[k] = "
                  << (A.d.access == OP2G_INC ? inc_zero(A.d.dtype) : "(" + std::string(T) + ")0")
                  << ";\n";
                kargs.push_back("op2g::ptr(t" + an + ")");
            }
        }
        if (S.loop.pass_layer_arg) kargs.push_back("layer");
        if (declared_without_parameters(S.user_src, S.kernel_name)) kargs.clear();
        // Call (pyop2/codegen/builder.py:964-977)
        O << J << S.kernel_name << "(";
        for (size_t i = 0; i < kargs.size(); ++i) O << (i ? ", " : "") << kargs[i];
        O << ");\n";

        // Unpacks (pyop2/codegen/builder.py:283-300, 386-410, 554-606)
        if (guard_unpack) O << J << "if (active) {\n";
        for (size_t a = 0; a < S.args.size(); ++a) {
            const ArgInfo &A = S.args[a];
            const char *T = ctype_of(A.d.dtype);
            const std::string an = std::to_string(a);
            if (A.d.kind == OP2G_ARG_GLOBAL) {
                if (A.d.access == OP2G_INC)
                    O << J << "for (int j = 0; j < " << A.d.dim << "; ++j) gacc" << an << "[j] += g"
                      << an << "[j];\n";
                else if (A.d.access == OP2G_MIN)
                    O << J << "for (int j = 0; j < " << A.d.dim << "; ++j) gacc" << an
                      << "[j] = op2g::vmin(gacc" << an << "[j], g" << an << "[j]);\n";
                else if (A.d.access == OP2G_MAX)
                    O << J << "for (int j = 0; j < " << A.d.dim << "; ++j) gacc" << an
                      << "[j] = op2g::vmax(gacc" << an << "[j], g" << an << "[j]);\n";
            } else if (A.d.kind == OP2G_ARG_DAT && A.d.map >= 0 && A.d.access != OP2G_READ) {
                const int ar = S.maps[A.d.map].arity;
                const int D = A.d.dim;
                if (warp && A.d.access == OP2G_INC) {
                    for (int f = 0; f < nf; ++f)
                        O << J << "for (int i = 0; i < " << ar << "; ++i) ti" << an << "[" << f * ar
                          << " + i] = " << idx_arr(A.d.map, f) << "[i];\n";
                    continue;  // scattered after the active block
                }
                if (staging && st_arg[a] >= 0) {
                    // staged INC: each entry owns its slot (plain store); the
                    // slots of one target are summed when the partition is done
                    O << J << "#pragma unroll\n";
                    O << J << "for (int i = 0; i < " << ar << "; ++i) {\n";
                    O << J << "  const int l_ = " << local_index(a, "i") << ";\n";
                    O << J << "  if (l_ == 0xFFFF) continue;\n";
                    O << J << "#pragma unroll\n";
                    O << J << "  for (int j = 0; j < " << D << "; ++j) sv" << a << "[l_ * " << D
                      << " + j] = t" << first[a] << "[" << poff[a] << " + i * " << D << " + j];\n";
                    O << J << "}\n";
                    continue;
                }
                O << J << "{ " << T << " *d_ = (" << T << " *)p.ptr[" << A.slot << "];\n";
                for (int f = 0; f < nf; ++f) {
                    O << J << "#pragma unroll\n";
                    O << J << "  for (int i = 0; i < " << ar << "; ++i) {\n";
                    O << J << "    const int x_ = " << idx_arr(A.d.map, f) << "[i];\n";
                    O << J << "    if (x_ < 0) continue;\n";
                    if (shared_ts[a]) {
                        // find or claim x_'s slot (bounded linear probing;
                        // a full table sends the contribution to global memory)
                        const int TS = shared_ts[a];
                        O << J << "    int h_ = (int)(((unsigned)x_ * 2654435761u) & " << TS - 1
                          << "u);\n";
                        O << J << "    for (int q_ = 0; ; ++q_) {\n";
                        O << J << "      if (q_ == " << TS << ") { h_ = -1; break; }\n";
                        O << J << "      const int o_ = atomicCAS(&sk" << a << "[h_], -1, x_);\n";
                        O << J << "      if (o_ == -1) { sl" << a << "[atomicAdd(&sn" << a
                          << "[par_], 1)] = h_; break; }\n";
                        O << J << "      if (o_ == x_) break;\n";
                        O << J << "      h_ = (h_ + 1) & " << TS - 1 << ";\n";
                        O << J << "    }\n";
                    }
                    O << J << "#pragma unroll\n";
                    O << J << "    for (int j = 0; j < " << D << "; ++j) {\n";
                    std::string dst = "d_[(long long)x_ * " + std::to_string(gstride(a)) + " + j]";
                    std::string src = "t" + std::to_string(first[a]) + "[" +
                                      std::to_string(poff[a]) + " + (" + std::to_string(f * ar) +
                                      " + i) * " + std::to_string(D) + " + j]";
                    switch (A.d.access) {
                        case OP2G_INC:
                            if (plain) O << J << "      " << dst << " += " << src << ";\n";
                            else if (shared_ts[a])
                                O << J << "      if (h_ >= 0) op2g::atomic_inc(&sv" << a << "[h_ * "
                                  << D << " + j], " << src << "); else op2g::atomic_inc(&" << dst
                                  << ", " << src << ");\n";
                            else O << J << "      op2g::atomic_inc(&" << dst << ", " << src << ");\n";
                            break;
                        case OP2G_MIN:
                            if (plain) O << J << "      " << dst << " = op2g::vmin(" << dst << ", " << src << ");\n";
                            else O << J << "      op2g::atomic_min(&" << dst << ", " << src << ");\n";
                            break;
                        case OP2G_MAX:
                            if (plain) O << J << "      " << dst << " = op2g::vmax(" << dst << ", " << src << ");\n";
                            else O << J << "      op2g::atomic_max(&" << dst << ", " << src << ");\n";
                            break;
                        default:  // WRITE, RW
                            O << J << "      " << dst << " = " << src << ";\n";
                    }
                    O << J << "    }\n";
                    O << J << "  }\n";
                }
                O << J << "}\n";
            } else if (A.d.kind == OP2G_ARG_MAT) {
                // MatSetValuesBlockedLocal(ADD|INSERT) on block-CSR storage.
                const int ra = S.maps[A.d.map].arity, ca = S.maps[A.d.cmap].arity;
                const int RD = A.d.rdim, CD = A.d.cdim;
                const int ncolv = rstride[a];
                const std::string tn = "t" + std::to_string(first[a]);
                O << J << "{ " << T << " *v_ = (" << T << " *)p.ptr[" << A.slot << "];\n";
                O << J << "  const long long *rp_ = (const long long *)p.ptr[" << A.slot + 1 << "];\n";
                O << J << "  const int *ci_ = (const int *)p.ptr[" << A.slot + 2 << "];\n";
                for (int fr = 0; fr < nf; ++fr)
                    for (int fc = 0; fc < nf; ++fc) {
                        O << J << "  for (int i = 0; i < " << ra << "; ++i) {\n";
                        O << J << "    const int r_ = " << idx_arr(A.d.map, fr) << "[i];\n";
                        O << J << "    if (r_ < 0) continue;\n";
                        O << J << "    for (int j = 0; j < " << ca << "; ++j) {\n";
                        O << J << "      const int c_ = " << idx_arr(A.d.cmap, fc) << "[j];\n";
                        O << J << "      if (c_ < 0) continue;\n";
                        O << J << "      const long long q_ = op2g::bcsr_find(rp_, ci_, r_, c_);\n";
                        O << J << "      if (q_ < 0) { op2g::set_err(p.err, OP2G_DEVERR_NEW_NONZERO); continue; }\n";
                        O << J << "#pragma unroll\n";
                        O << J << "      for (int ri = 0; ri < " << RD << "; ++ri)\n";
                        O << J << "#pragma unroll\n";
                        O << J << "        for (int cj = 0; cj < " << CD << "; ++cj) {\n";
                        O << J << "          const " << T << " w_ = " << tn << "[(" << roff[a]
                          << " + (" << fr * ra << " + i) * " << RD << " + ri) * " << ncolv << " + "
                          << coff[a] << " + (" << fc * ca << " + j) * " << CD << " + cj];\n";
                        std::string dst = "v_[q_ * " + std::to_string(RD * CD) + " + ri * " +
                                          std::to_string(CD) + " + cj]";
                        if (A.d.access == OP2G_INC) {
                            if (plain) O << J << "          " << dst << " += w_;\n";
                            else O << J << "          op2g::atomic_inc(&" << dst << ", w_);\n";
                        } else {
                            O << J << "          " << dst << " = w_;\n";
                        }
                        O << J << "        }\n";
                        O << J << "    }\n";
                        O << J << "  }\n";
                    }
                O << J << "}\n";
            }
        }
        if (guard_unpack) O << J << "}\n";
    }
};

// Validate a signature; returns an error message or "".
std::string validate_signature(const Signature &S) {
    if (S.kernel_name.empty()) return "empty kernel name";
    for (size_t m = 0; m < S.maps.size(); ++m) {
        const MapInfo &mi = S.maps[m];
        if (mi.arity <= 0) return "map " + std::to_string(m) + ": arity must be positive";
        if (mi.kind == OP2G_MAP_PERMUTED) {
            if (mi.base < 0 || mi.base >= (int)S.maps.size() || S.maps[mi.base].kind != OP2G_MAP_PLAIN)
                return "map " + std::to_string(m) + ": permuted map must refer to a plain map";
            if ((int)mi.permutation.size() != mi.arity) return "permutation length != arity";
        } else if (mi.kind == OP2G_MAP_COMPOSED) {
            if (mi.ncomposed < 2 || mi.ncomposed > OP2G_MAX_COMPOSED) return "bad composed chain";
            for (int k = 0; k < mi.ncomposed; ++k) {
                int c = mi.composed[k];
                if (c < 0 || c >= (int)S.maps.size() || S.maps[c].kind == OP2G_MAP_COMPOSED)
                    return "composed chain must refer to plain or permuted maps (flatten first)";
                if (k >= 1 && S.maps[c].arity != 1) return "inner maps of a composition need arity 1";
            }
        } else if (mi.kind != OP2G_MAP_PLAIN) {
            return "unknown map kind";
        }
    }
    for (size_t a = 0; a < S.args.size(); ++a) {
        const op2g_arg_desc &d = S.args[a].d;
        std::string an = "argument " + std::to_string(a) + ": ";
        if (!ctype_of(d.dtype)) return an + "unknown dtype";
        if (d.access < OP2G_READ || d.access > OP2G_MAX) return an + "unknown access";
        switch (d.kind) {
            case OP2G_ARG_DAT:
                if (d.dim <= 0) return an + "dim must be positive";
                if (d.stride < 0 || (d.stride > 0 && d.stride < d.dim))
                    return an + "stride must be 0 or at least dim";
                if (d.map >= (int)S.maps.size()) return an + "map index out of range";
                if (d.map >= 0 && (d.access == OP2G_INC || d.access == OP2G_MIN || d.access == OP2G_MAX) &&
                    !atomic_capable(d.dtype) && S.loop.scatter != OP2G_SCATTER_PLAIN)
                    return an + "INC/MIN/MAX through a map needs a 32- or 64-bit element type";
                break;
            case OP2G_ARG_GLOBAL:
                if (d.dim <= 0) return an + "dim must be positive";
                if (d.access != OP2G_READ && d.access != OP2G_INC && d.access != OP2G_MIN &&
                    d.access != OP2G_MAX)
                    return an + "Globals take READ, INC, MIN or MAX";
                if (d.access != OP2G_READ && !atomic_capable(d.dtype))
                    return an + "Global reductions need a 32- or 64-bit element type";
                break;
            case OP2G_ARG_MAT:
                if (d.access != OP2G_INC && d.access != OP2G_WRITE) return an + "Mats take INC or WRITE";
                if (d.map < 0 || d.cmap < 0 || d.map >= (int)S.maps.size() || d.cmap >= (int)S.maps.size())
                    return an + "Mat needs row and column maps";
                if (d.rdim <= 0 || d.cdim <= 0) return an + "bad Mat block dims";
                if (!atomic_capable(d.dtype)) return an + "Mat values need a 32- or 64-bit type";
                break;
            case OP2G_ARG_PASSTHROUGH:
                break;
            default:
                return an + "unknown kind";
        }
    }
    // Groups (mixed arguments): contiguous, homogeneous, consistent block shapes.
    for (size_t a = 0; a < S.args.size();) {
        const op2g_arg_desc &d0 = S.args[a].d;
        if (d0.group < 0) return "argument " + std::to_string(a) + ": negative group id";
        size_t b = a + 1;
        if (d0.group > 0) {
            while (b < S.args.size() && S.args[b].d.group == d0.group) ++b;
            for (size_t k = b; k < S.args.size(); ++k)
                if (S.args[k].d.group == d0.group)
                    return "group " + std::to_string(d0.group) + " is not contiguous";
            for (size_t k = a; k < b; ++k) {
                const op2g_arg_desc &d = S.args[k].d;
                std::string an = "argument " + std::to_string(k) + ": ";
                if (d.kind != d0.kind || d.access != d0.access || d.dtype != d0.dtype)
                    return an + "grouped arguments need one kind, access and dtype";
                if (d.kind == OP2G_ARG_DAT && d.map < 0)
                    return an + "grouped Dat components must be indirect";
                if (d.kind != OP2G_ARG_DAT && d.kind != OP2G_ARG_MAT)
                    return an + "only Dats and Mats can be grouped";
                if (d.kind == OP2G_ARG_MAT && d.group_cols != d0.group_cols)
                    return an + "group_cols differs within the group";
            }
            if (d0.kind == OP2G_ARG_MAT) {
                const int C = d0.group_cols;
                if (C <= 0 || (b - a) % (size_t)C != 0)
                    return "argument " + std::to_string(a) + ": group_cols must divide the block count";
                auto rows = [&](size_t k) {
                    const op2g_arg_desc &d = S.args[k].d;
                    return S.maps[d.map].arity * d.rdim;
                };
                auto cols = [&](size_t k) {
                    const op2g_arg_desc &d = S.args[k].d;
                    return S.maps[d.cmap].arity * d.cdim;
                };
                for (size_t k = a; k < b; ++k) {
                    size_t i = (k - a) / C, j = (k - a) % C;
                    if (rows(k) != rows(a + i * C) || cols(k) != cols(a + j))
                        return "argument " + std::to_string(k) + ": block shape does not match its block row/column";
                }
            }
        }
        a = b;
    }
    if (S.loop.pass_layer_arg && !S.loop.extruded) return "layer argument needs an extruded loop";
    if (S.loop.scatter < OP2G_SCATTER_ATOMIC || S.loop.scatter > OP2G_SCATTER_STAGED)
        return "unknown scatter strategy";
    return "";
}

// Alignment of every row of direct Dat argument a when its array is
// aligned to it: 32 or 16 bytes for rows of a multiple of that size, else 0.
int direct_row_alignment(const Signature &S, size_t a) {
    const op2g_arg_desc &d = S.args[a].d;
    if (d.kind != OP2G_ARG_DAT || d.map >= 0) return 0;
    const long long rb = (long long)(d.stride > 0 ? d.stride : d.dim) * (long long)elt_size(d.dtype);
    return rb % 32 == 0 ? 32 : rb % 16 == 0 ? 16 : 0;
}

std::vector<std::pair<int, int>> aligned_direct_args(const Signature &S) {
    std::vector<std::pair<int, int>> out;
    for (int r : staged_args(S))
        if (r >= 0) return out;
    for (size_t a = 0; a < S.args.size(); ++a) {
        const int al = direct_row_alignment(S, a);
        if (al) out.push_back({S.args[a].slot, al});
    }
    return out;
}

std::string generate_source(const Signature &S, int *cells_per_thread, bool align_hints) {
    Gen g(S);
    g.align_hints = align_hints;
    std::string src = g.emit();
    if (cells_per_thread) *cells_per_thread = g.cells_per_thread;
    return src;
}

}  // namespace op2g
