/*
 * op2g.h -- C ABI of libop2g, the GB300 (sm_103a) execution engine behind the
 * PyOP2-compatible Python package `pyop2_gb300`.
 *
 * Everything here is plain C: integers, sizes and raw pointers.  Device
 * pointers are CUDA global-memory addresses on the current device; "stream"
 * is a cudaStream_t passed as void* (NULL = legacy default stream).  No call
 * allocates device memory except where stated; callers own every buffer.
 *
 * Every entry point returns an op2g_status (0 = success).  On failure the
 * thread-local message returned by op2g_last_error() says why.
 *
 * Which reference interface each group replaces (paths inside PyOP2 0.12.0):
 *   op2g_kernel_*      the JIT-compiled, ctypes-called sequential wrapper
 *                      `wrap_<name>(start, end, [layers], [subset], args..., maps...)`
 *                      produced by pyop2/global_kernel.py:364-417 (compile/argtypes)
 *                      from pyop2/codegen/builder.py:683-989 (WrapperBuilder) and
 *                      called at pyop2/global_kernel.py:322-331.
 *   op2g_sparsity_*    pyop2/sparsity.pyx:121-175 (build_sparsity) and
 *                      pyop2/sparsity.pyx:178-405 (fill_with_zeros), which walk
 *                      Map pairs into a PETSc MATPREALLOCATOR.
 *   op2g_mat_*         the PETSc calls behind pyop2/types/mat.py: zeroEntries
 *                      (:786-790), zeroRowsLocal (:792-801), setValuesLocalRCV
 *                      for set_local_diagonal_entries (:806-827), MatMult for
 *                      Mat * vector (:850-855 in the abstract interface).
 *   op2g_colour_*      the two-level greedy colouring "plan" of the historical
 *                      OP2 CUDA backend, documented in doc/sphinx/source/plan.rst:43-80
 *                      (no code counterpart in this checkout).
 */
#ifndef OP2G_H
#define OP2G_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define OP2G_ABI_VERSION 4

/* ---------------------------------------------------------------- status */
typedef int32_t op2g_status;
enum {
    OP2G_OK = 0,
    OP2G_ERR_INVALID = 1,      /* bad argument / descriptor                     */
    OP2G_ERR_COMPILE = 2,      /* NVRTC rejected the generated source           */
    OP2G_ERR_CUDA = 3,         /* a CUDA runtime/driver call failed             */
    OP2G_ERR_BOUNDS = 4,       /* a device-side check tripped (map out of range) */
    OP2G_ERR_NEW_NONZERO = 5,  /* Mat insertion outside the sparsity pattern    */
    OP2G_ERR_CAPACITY = 6,     /* a fixed device capacity was exceeded          */
    OP2G_ERR_UNSUPPORTED = 7,  /* feature not implemented                       */
    OP2G_ERR_TIMEOUT = 8       /* a bounded device wait gave up                 */
};

/* Device-side error word bits (written with atomicOr by generated kernels). */
enum {
    OP2G_DEVERR_MAP_BOUNDS = 1,   /* map value >= toset size (debug builds)  */
    OP2G_DEVERR_NEW_NONZERO = 2,  /* (row, col) not in the Mat's pattern     */
    OP2G_DEVERR_CAPACITY = 4,     /* row candidate list above the capacity   */
    OP2G_DEVERR_TIMEOUT = 8       /* a bounded wait of a staged wrapper gave up */
};

/* Thread-local description of the last failure (never NULL). */
const char *op2g_last_error(void);
/* OP2G_ABI_VERSION of the loaded library. */
int32_t op2g_abi_version(void);

/* Make `device` current for this thread and initialise its primary context.
 * Returns the SM count and compute capability through the out-pointers
 * (either may be NULL). */
op2g_status op2g_device_init(int32_t device, int32_t *sm_count, int32_t *cc_major,
                             int32_t *cc_minor);

/* ---------------------------------------------------- par_loop wrappers */
/* Access descriptors: same integer values as pyop2/types/access.py:4-10. */
enum { OP2G_READ = 1, OP2G_WRITE = 2, OP2G_RW = 3, OP2G_INC = 4, OP2G_MIN = 5, OP2G_MAX = 6 };
/* Iteration regions: same values as pyop2/types/__init__.py:14-18. */
enum { OP2G_ON_BOTTOM = 1, OP2G_ON_TOP = 2, OP2G_ON_INTERIOR_FACETS = 3, OP2G_ALL = 4 };
/* Element types (numpy dtype -> C type, pyop2/datatypes.py:13-29). */
enum {
    OP2G_F64 = 0, OP2G_F32 = 1, OP2G_I32 = 2, OP2G_U32 = 3, OP2G_I64 = 4, OP2G_U64 = 5,
    OP2G_I16 = 6, OP2G_U16 = 7, OP2G_I8 = 8, OP2G_U8 = 9
};
/* Argument kinds (pyop2/global_kernel.py:89-247). */
enum { OP2G_ARG_DAT = 0, OP2G_ARG_GLOBAL = 1, OP2G_ARG_MAT = 2, OP2G_ARG_PASSTHROUGH = 3 };
/* Map kinds (pyop2/types/map.py: Map :17, PermutedMap :171, ComposedMap :218). */
enum { OP2G_MAP_PLAIN = 0, OP2G_MAP_PERMUTED = 1, OP2G_MAP_COMPOSED = 2 };
/* How INC contributions to indirect Dats and Mats reach memory. */
enum {
    OP2G_SCATTER_ATOMIC = 0,   /* one hardware atomic (RED) per contribution          */
    OP2G_SCATTER_WARP = 1,     /* __match_any_sync groups lanes on one target, one
                                  shuffle-reduced atomic per group                    */
    OP2G_SCATTER_PLAIN = 2,    /* plain read-modify-write: only legal when the caller
                                  launches one colour (conflict-free cell set) at a time */
    OP2G_SCATTER_SHARED = 3,   /* each CTA sums its INC contributions per target in a
                                  shared-memory hash table, then adds each distinct
                                  target once with a global atomic (non-extruded loops;
                                  atomics elsewhere)                                    */
    OP2G_SCATTER_STAGED = 4    /* the loop runs on a staging plan (op2g_stage_plan_*):
                                  per mini-partition, the data of READ Dat arguments
                                  through plain or permuted maps are staged in shared
                                  memory once per distinct target, INC contributions
                                  are stored at their entries' slots there, summed per
                                  target in slot order, and each distinct target
                                  receives one global atomic per partition
                                  (non-extruded, non-indexed loops; the launch passes the
                                  plan in op2g_launch_desc.stage; grid 0 = one resident
                                  wave whose CTAs pipeline their partitions, -1 = one
                                  CTA per partition)                                   */
};

#define OP2G_MAX_ARGS 32
#define OP2G_MAX_MAPS 32
#define OP2G_MAX_COMPOSED 8

/* One map of the loop.  Host arrays are copied during op2g_kernel_create and
 * baked into the generated code as constants (as the reference bakes map
 * offsets as named literals, pyop2/codegen/builder.py:55-62).
 * The device array of a plain map (int32 [entities, arity], row-major, passed
 * in the launch's pointer slots) must be 16-byte aligned when arity is a
 * multiple of 4 and 8-byte aligned when it is even: rows are read with
 * vector loads, and every launch checks the alignment.  It must not change
 * while a launch runs. */
typedef struct op2g_map_desc {
    int32_t kind;          /* OP2G_MAP_*                                                */
    int32_t arity;
    int32_t base;          /* PERMUTED: index of the permuted map in this table         */
    int32_t ncomposed;     /* COMPOSED: number of maps in `composed`                    */
    int32_t composed[OP2G_MAX_COMPOSED]; /* COMPOSED: maps_[0..ncomposed) (outermost first) */
    const int32_t *offset;          /* host, arity entries, or NULL (not extruded)     */
    const int32_t *offset_quotient; /* host, arity entries, or NULL                    */
    const int32_t *permutation;     /* host, arity entries (PERMUTED only)             */
} op2g_map_desc;

/* One argument of the loop, in kernel-argument order. */
typedef struct op2g_arg_desc {
    int32_t kind;     /* OP2G_ARG_*                                                  */
    int32_t access;   /* OP2G_READ .. OP2G_MAX                                       */
    int32_t dtype;    /* OP2G_F64 ..                                                 */
    int32_t dim;      /* DAT/GLOBAL: values per entity (cdim)                        */
    int32_t map;      /* DAT: map index or -1 (direct); MAT: row map index           */
    int32_t cmap;     /* MAT: column map index                                       */
    int32_t rdim;     /* MAT: rows per block                                          */
    int32_t cdim;     /* MAT: columns per block                                       */
    int32_t group;    /* 0, or an id > 0 shared by CONSECUTIVE arguments that form one
                         kernel parameter: the components of a MixedDat (their packs
                         concatenated in order, pyop2/codegen/builder.py:413-498) or the
                         blocks of a mixed Mat in row-major block order (one element
                         matrix over all blocks, pyop2/codegen/builder.py:609-680)      */
    int32_t group_cols; /* MAT groups: number of block columns                         */
    int32_t stride;   /* DAT: elements from one entity's values to the next (0 = dim).  A
                         view of one component of a dim-S Dat (DatView,
                         pyop2/types/dat.py:668-760) has dim 1, stride S, and its device
                         pointer at the component                                       */
} op2g_arg_desc;

typedef struct op2g_loop_desc {
    int32_t extruded;          /* iterate (entity, layer)                                 */
    int32_t constant_layers;   /* layers array has one row                                */
    int32_t extruded_periodic;
    int32_t indexed;           /* iterate indices[start..end) (Subset, colour order)      */
    int32_t iteration_region;  /* OP2G_ALL ..                                             */
    int32_t pass_layer_arg;    /* append `int layer` to the kernel call                   */
    int32_t scatter;           /* OP2G_SCATTER_*                                          */
    int32_t block_size;        /* threads per CTA (0 = 256)                               */
    int32_t debug_checks;      /* bounds-check every map value, report via error word     */
    int32_t batched;           /* build the persistent multi-loop variant (see _batch)    */
    int32_t prefetch;          /* 1: each thread loads the map rows (and subset index) of
                                  its next iteration before running the current one
                                  (non-extruded loops; more memory-level parallelism)   */
    int32_t nc_reads;          /* 1: READ Dat gathers use the read-only data path; the
                                  caller guarantees that no argument of the loop writes
                                  a Dat that a READ argument reads                      */
    int32_t cells_per_thread;  /* > 1: each thread runs that many iterations per sweep
                                  step, their gathers and arithmetic interleaved (an
                                  iteration past the end recomputes the last one and
                                  skips its unpack); loops with direct RW/INC/MIN/MAX
                                  or passthrough arguments, warp or shared-memory
                                  scatter or prefetch run one                          */
} op2g_loop_desc;

typedef struct op2g_kernel op2g_kernel;

/* Generate the CUDA wrapper around `user_src` (a C kernel whose entry point is
 * `kernel_name`), compile it with NVRTC for `arch` ("sm_103a"; NULL = the
 * current device) and return a handle.  `cache_dir` (may be NULL) holds
 * compiled cubins keyed by a hash of source, options and arch.  No device is
 * needed unless arch is NULL.  On OP2G_ERR_COMPILE op2g_last_error() holds
 * the NVRTC log.  When a direct DAT argument's rows are a multiple of 16
 * bytes (stride, or dim, x element size), a second variant is compiled that
 * declares every such row 16- or 32-byte aligned, so the kernel's accesses
 * to adjacent components become vector loads and stores; op2g_kernel_launch
 * runs it when all those arguments' pointers are aligned, the first variant
 * otherwise (batched launches always run the first). */
op2g_status op2g_kernel_create(const char *user_src, const char *kernel_name,
                               const op2g_loop_desc *loop, const op2g_arg_desc *args,
                               int32_t nargs, const op2g_map_desc *maps, int32_t nmaps,
                               const char *arch, const char *cache_dir, op2g_kernel **out);
void op2g_kernel_destroy(op2g_kernel *k);

/* Copy the generated CUDA source (the variant without alignment hints) into
 * buf (NUL-terminated, truncated to len); *needed receives strlen+1. */
op2g_status op2g_kernel_source(const op2g_kernel *k, char *buf, size_t len, size_t *needed);
/* Load the compiled wrapper (both variants) on the current device without
 * launching it.  Launches load it on first use; call this first when the
 * first launch will happen inside a CUDA stream capture (module loading is
 * not capturable). */
op2g_status op2g_kernel_prepare(op2g_kernel *k);
/* Number of device-pointer slots op2g_kernel_launch expects in `ptrs`:
 *   per argument, in order: DAT 1 (data), GLOBAL 1 (data, or the zeroed
 *   reduction temporary for INC), MAT 3 (values, rowptr int64, colidx int32),
 *   PASSTHROUGH 1; then one slot per map of the map table (values, int32
 *   [iterset total, arity], NULL for PERMUTED/COMPOSED entries). */
int32_t op2g_kernel_num_ptrs(const op2g_kernel *k);
/* Registers per thread of the loaded kernel (-1 before first launch). */
int32_t op2g_kernel_num_regs(const op2g_kernel *k);

/* The staging plan of a launch of a wrapper built with OP2G_SCATTER_STAGED:
 * the iteration range is cut into mini-partitions of `block` iterations
 * (partition p = [p * block, (p + 1) * block)).  For every map of the map
 * table that the plan covers (entry m; a permuted map uses its base map's
 * entry), partition p's segment starts at ind_off[m][p] (a multiple of 8)
 * and holds ind_num[m][p] distinct targets in ascending order
 * (ind_map[m] + ind_off[m][p] ...) with the first slot of each in
 * run_off[m] + ind_off[m][p] (followed by the partition's count of valid
 * entries); loc_map[m][i * arity + j] is entry (i, j)'s slot: its rank in the
 * partition's entries sorted by (target, position), 0xFFFF for a negative
 * entry.  Built by op2g_stage_plan_count / _fill; all arrays on the device. */
typedef struct op2g_stage_desc {
    int64_t block;
    int64_t n;                          /* iterations the plan covers: [0, n)      */
    const int32_t *ind_map[OP2G_MAX_MAPS];
    const int64_t *ind_off[OP2G_MAX_MAPS];
    const int32_t *ind_num[OP2G_MAX_MAPS];
    const uint16_t *run_off[OP2G_MAX_MAPS];
    const uint16_t *loc_map[OP2G_MAX_MAPS];
    int32_t max_unique[OP2G_MAX_MAPS];  /* largest distinct count of a partition */
} op2g_stage_desc;

typedef struct op2g_launch_desc {
    int64_t start, end;        /* iteration range (entities; indices range if indexed)    */
    const int32_t *layers;     /* device layers array [*, 2] (extruded) or NULL          */
    const int32_t *indices;    /* device entity indices (indexed) or NULL                */
    int32_t *err;              /* device error word (OP2G_DEVERR_* bits) or NULL         */
    void *const *ptrs;         /* host array of op2g_kernel_num_ptrs device pointers     */
    const int64_t *map_toset;  /* host array, toset size per map (bounds checks) or NULL */
    int64_t layers_per_entity; /* constant-layer extrusion: layers iterated per entity,
                                  used only to size the grid (0 = 1)                     */
    int32_t grid;              /* CTAs.  0: one per block_size iterations, at most 4 x the
                                  CTAs the GPU holds at once (threads then stride over
                                  the rest); a launch of fewer than 4 full CTAs per SM
                                  instead runs k CTAs per SM on equal contiguous chunks,
                                  with fewer threads per CTA when a chunk is small
                                  (wrappers without shared-memory staging);
                                  -1: one per block_size iterations, no cap;
                                  > 0: exactly this many                               */
    const op2g_stage_desc *stage; /* OP2G_SCATTER_STAGED wrappers: the plan (host struct,
                                     read during the call); NULL otherwise             */
} op2g_launch_desc;

/* Launch the wrapper over [start, end) on `stream`.  Asynchronous. */
op2g_status op2g_kernel_launch(op2g_kernel *k, const op2g_launch_desc *d, void *stream);
/* The launch shape op2g_kernel_launch uses (pure function, no device use):
 * `items` iterations over `entities` entities, a wrapper compiled for
 * `block_size` threads holding `ctas_per_sm` CTAs on each of `sms` SMs,
 * the descriptor's `grid` request, and whether the wrapper has the balanced
 * entry (wrappers without shared-memory staging).  Outputs CTAs, threads
 * per CTA and 1 when the balanced entry runs. */
void op2g_launch_shape(int64_t items, int64_t entities, int32_t block_size, int32_t sms,
                       int32_t ctas_per_sm, int32_t grid_request, int32_t chunked_available,
                       int32_t *grid_out, int32_t *block_out, int32_t *chunked_out);

/* Persistent batched launch of a kernel built with loop->batched = 1: one
 * launch runs nloops loops of the same signature.  `params` is a DEVICE array
 * of nloops records, each op2g_kernel_param_bytes(k) bytes, laid out as
 * op2g_kernel_pack_params writes them; `work` is a DEVICE array of nwork
 * (loop index, start, end) int64 triples.  CTAs take work items round robin. */
int32_t op2g_kernel_param_bytes(const op2g_kernel *k);
op2g_status op2g_kernel_pack_params(const op2g_kernel *k, const op2g_launch_desc *d,
                                    void *out_host_record);
op2g_status op2g_kernel_launch_batched(op2g_kernel *k, const void *params_dev,
                                       const int64_t *work_dev, int64_t nwork,
                                       int32_t grid, void *stream);

/* CUDA graphs of op2g launches: record a step once, replay it with one call
 * (the reference builds no graphs; here several par_loops, or one batched
 * launch of many, run as one unit).  op2g_graph_begin returns a private
 * stream in capture mode; launch on it with op2g_kernel_launch,
 * op2g_kernel_launch_batched, op2g_mat_spmv, ... (call op2g_kernel_prepare
 * for each kernel first: module loading is not capturable; nothing on the
 * capture stream runs until the graph is launched).  op2g_graph_end always
 * ends the capture and releases the stream; it instantiates the recorded
 * graph into *out.  Device arrays the launches referenced are used, not
 * copied, by every replay and must outlive the graph. */
typedef struct op2g_graph op2g_graph;
op2g_status op2g_graph_begin(void **capture_stream);
op2g_status op2g_graph_end(void *capture_stream, op2g_graph **out);
/* Replay on `stream` (asynchronous). */
op2g_status op2g_graph_launch(op2g_graph *g, void *stream);
void op2g_graph_destroy(op2g_graph *g);

/* ------------------------------------------------------------- sparsity */
/* One (row map, column map, iteration region) triple of a Sparsity
 * (pyop2/types/mat.py:118-176).  Map arrays are device int32
 * [nent_total, arity]; composed chains are device pointers to arity-1 maps,
 * applied innermost-last as in pyop2/sparsity.pyx:249-259. */
typedef struct op2g_sparsity_pair {
    const int32_t *rmap, *cmap;
    int32_t rarity, carity;
    int64_t nent;                 /* entities iterated (iterset.size)                 */
    int32_t region;               /* OP2G_ALL ..                                      */
    int32_t nrcomposed, nccomposed;
    const int32_t *rcomposed[OP2G_MAX_COMPOSED];
    const int32_t *ccomposed[OP2G_MAX_COMPOSED];
    const int32_t *roffset, *coffset;                   /* host, or NULL          */
    const int32_t *roffset_quotient, *coffset_quotient; /* host, or NULL          */
} op2g_sparsity_pair;

typedef struct op2g_sparsity_desc {
    int64_t nrows, ncols;         /* block rows / block columns                      */
    int32_t set_diag;             /* add (i, i) for i < min(nrows, ncols)            */
    int32_t extruded, constant_layers, extruded_periodic;
    const int32_t *layers;        /* device layers array of the iterset (extruded)   */
    int32_t layer_slots;          /* extruded: max over entities of layers[e,1] - layers[e,0]
                                     (an upper bound of cells per column)             */
    int32_t npairs;
    const op2g_sparsity_pair *pairs;
} op2g_sparsity_desc;

/* Bytes of device workspace op2g_sparsity_build needs for `d`. */
op2g_status op2g_sparsity_workspace(const op2g_sparsity_desc *d, size_t *bytes);
/* Phase 1: rowptr[nrows+1] (int64, device) gets the exclusive prefix sum of
 * the per-row counts of distinct columns; *nnz (host) the total.  The call
 * synchronises `stream` to return nnz. */
op2g_status op2g_sparsity_count(const op2g_sparsity_desc *d, void *workspace, size_t ws_bytes,
                                int64_t *rowptr, int64_t *nnz, void *stream);
/* Phase 2: colidx[nnz] (int32, device) receives each row's columns, sorted
 * ascending and unique.  Must follow op2g_sparsity_count with the same
 * workspace (it reuses the row->entity transpose kept there). */
op2g_status op2g_sparsity_fill(const op2g_sparsity_desc *d, void *workspace, size_t ws_bytes,
                               const int64_t *rowptr, int32_t *colidx, void *stream);

/* ------------------------------------------------------- staging plans */
/* The staging plan of one map over n iterations in partitions of `block`
 * iterations (block * arity <= 4096): the local renumbering of the
 * historical OP2 execution plan, doc/sphinx/source/plan.rst:21-39 (no code
 * counterpart in this checkout), with one slot per map entry in place of that
 * plan's thread colouring.  `map` is the device int32 [n, arity] array.
 * op2g_stage_plan_count writes ind_off[nblocks + 1] (device int64, exclusive
 * prefix sums of the segment lengths: distinct count + 1 rounded up to 8) and
 * ind_num[nblocks] (device int32, distinct counts), and returns the total
 * segment length and the largest distinct count (synchronises `stream`);
 * op2g_stage_plan_fill then writes ind_map[total] (int32), run_off[total]
 * (uint16) and loc_map[n * arity] (uint16), all device arrays.  workspace:
 * op2g_stage_plan_workspace bytes of device memory. */
op2g_status op2g_stage_plan_workspace(int64_t n, int32_t arity, int64_t block, size_t *bytes);
op2g_status op2g_stage_plan_count(int64_t n, int32_t arity, const int32_t *map, int64_t block,
                                  void *workspace, size_t ws_bytes, int64_t *ind_off,
                                  int32_t *ind_num, int64_t *total, int32_t *max_unique,
                                  void *stream);
op2g_status op2g_stage_plan_fill(int64_t n, int32_t arity, const int32_t *map, int64_t block,
                                 const int64_t *ind_off, int32_t *ind_map, uint16_t *run_off,
                                 uint16_t *loc_map, void *stream);

/* ----------------------------------------------------------- matrices */
/* Block-CSR matrix with rdim x cdim row-major blocks (rdim = cdim = 1 is CSR). */
typedef struct op2g_bcsr {
    int64_t nrows, ncols;      /* block rows / block columns */
    int32_t rdim, cdim;
    const int64_t *rowptr;     /* device [nrows + 1] */
    const int32_t *colidx;     /* device [nnz]       */
    double *values;            /* device [nnz * rdim * cdim] */
} op2g_bcsr;

/* Zero the given dof rows (rows are dof indices: block_row * rdim + r) keeping
 * the pattern, and put diag_val on their diagonal (zeroRowsLocal). */
op2g_status op2g_mat_zero_rows(const op2g_bcsr *m, const int32_t *rows_dev, int64_t nrows_zero,
                               double diag_val, void *stream);
/* Set (INSERT) diag_val on the diagonal of the given dof rows. */
op2g_status op2g_mat_set_diagonal(const op2g_bcsr *m, const int32_t *rows_dev, int64_t n,
                                  double diag_val, int32_t *err, void *stream);
/* y = A x (transpose = 0) or y = A^T x (transpose = 1; y must be zeroed, uses atomics). */
op2g_status op2g_mat_spmv(const op2g_bcsr *m, const double *x, double *y, int32_t transpose,
                          void *stream);

/* ------------------------------------------------------------ colouring */
/* Greedy colouring of `ncells` entities so that no two entities of one colour
 * share a target through any of the `nmaps` maps (device int32 [ncells, arity_k],
 * negative values ignored).  Each target set has `target_size[k]` entries.
 * Outputs (device): colour[ncells] int32, order[ncells] int32 (entities sorted
 * by colour, stable), colour_ptr[max_colours + 1] int64 (segment offsets).
 * *ncolours (host) receives the colour count; the call synchronises.  Fails
 * with OP2G_ERR_CAPACITY if more than max_colours colours are needed.
 * workspace: op2g_colour_workspace bytes of device memory. */
op2g_status op2g_colour_workspace(int64_t ncells, int32_t nmaps, const int64_t *target_size,
                                  size_t *bytes);
op2g_status op2g_colour(int64_t ncells, int32_t nmaps, const int32_t *const *maps,
                        const int32_t *arity, const int64_t *target_size, int32_t max_colours,
                        void *workspace, size_t ws_bytes, int32_t *colour, int32_t *order,
                        int64_t *colour_ptr, int32_t *ncolours, void *stream);

/* Colouring without allocation (no counterpart in the reference).
 * For callers that cannot allocate device memory -- a host whose device
 * memory is owned by another allocator or a pool sized up front, or a runtime
 * that forbids cudaMalloc after start-up -- this is op2g_colour with its
 * scratch in a fixed device array of the library
 * (OP2G_COLOUR_NOALLOC_SCRATCH_BYTES, held by every GPU that loads the
 * library until the process exits) instead of a caller workspace.  Inputs
 * and outputs are the caller's, as for op2g_colour.  It calls no
 * cudaMalloc/cudaFree (nor any allocating library routine) and allocates no
 * host memory.  Like op2g_colour it reads a count back and synchronises
 * `stream` in every colouring round.
 * Problems whose op2g_colour_workspace size exceeds the array fail with
 * OP2G_ERR_CAPACITY.  The first call on a device looks up the array's device
 * address (cudaGetSymbolAddress, once per device, under a lock).  All calls
 * share the one array and each call clears what it needs: calls that overlap
 * on the GPU (different streams, or threads) race and must be serialised by
 * the caller. */
#define OP2G_COLOUR_NOALLOC_SCRATCH_BYTES (16 * 1024 * 1024)
#define OP2G_NOALLOC_MAX_DEVICES 64
op2g_status op2g_colour_noalloc(int64_t ncells, int32_t nmaps, const int32_t *const *maps,
                                const int32_t *arity, const int64_t *target_size,
                                int32_t max_colours, int32_t *colour, int32_t *order,
                                int64_t *colour_ptr, int32_t *ncolours, void *stream);

/* --------------------------------------------------------- measurement */
/* Time a register-resident FP64 FMA loop over the whole GPU and return the
 * achieved FP64 rate (flop/s, FMA = 2) -- the second roofline ceiling of the
 * element kernels.  Synchronous. */
op2g_status op2g_probe_fp64_peak(double *flops_per_s, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* OP2G_H */
