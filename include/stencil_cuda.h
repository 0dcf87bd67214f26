/*
 * stencil_cuda.h — C ABI of libstencilcuda.so, the GB300 (sm_103a) implementation of
 * Stencils.jl's `mapstencil` / `mapstencil!` hot path.
 *
 * Every entry point takes plain pointers and sizes.  Grids are column-major (axis 0 is the
 * contiguous one, exactly as a Julia `Array`), live in caller-owned device memory, and are
 * described by `stc_grid`.  The library never frees caller memory.  Its own scratch (packed Life
 * grids, padded pairs, batch tables) is stream-ordered memory from the device's default pool, whose
 * release threshold the library raises to 1 GiB on first use (a higher threshold the application set
 * stays), so scratch pages stay mapped across synchronisations; applications that share that pool
 * see it keep up to 1 GiB of freed memory.  Calls are ordered on the
 * CUDA stream passed as `void* stream` (a `cudaStream_t`; NULL is the legacy default stream).
 * Every call returns STC_OK (0) or a negative `stc_status`; `stc_strerror` names it.  The
 * statuses mirror the `ArgumentError`s the reference raises, so a Julia shim can rethrow them.
 *
 * Reference interfaces replaced (Stencils.jl v0.3.6, paths within the package):
 *   stc_map               gatherstencil!(f, dest, source::AbstractStencilArray)   src/gatherstencil.jl:89-103
 *                         (and gatherstencil(f, source), which allocates dest,   src/gatherstencil.jl:14-39)
 *   stc_map_steps         repeated  A = gatherstencil!(f, A::SwitchingStencilArray) src/gatherstencil.jl:77-83
 *                         with switch(A)                                        src/array.jl:610-611
 *   stc_map_terms         gatherstencil!(f, dest, source, args...) with several arrays, f a
 *                         registered sum of per-array terms                      src/gatherstencil.jl:84-113
 *   stc_scatter           scatterstencil!(f, op, dest, source) for registered f and op
 *                                                                                src/scatterstencil.jl:36-133
 *   stc_update_boundary   update_boundary!(A::AbstractStencilArray)              src/array.jl:195-233
 *   stc_mass              no counterpart: FP64 compensated total of a grid, used to report the mass
 *                         drift of long multi-step runs.
 *   stc_batch_*           no counterpart: many independent `mapstencil!` loops run as one
 *                         CUDA-graph-captured persistent launch.
 *   stc_server_*          no counterpart: a continuous-batching request loop over stc_batch.
 * `mapstencil` / `mapstencil!` are the deprecated aliases of the above (src/gatherstencil.jl:127-128).
 */
#ifndef STENCIL_CUDA_H
#define STENCIL_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define STC_API __attribute__((visibility("default")))
#else
#define STC_API
#endif

#define STC_ABI_VERSION 2

/* ---- status codes (the reference's ArgumentError sites in comments) ---- */
typedef enum {
    STC_OK = 0,
    STC_ERR_SIZE_MISMATCH = -1,   /* "Source array sizes must match"  src/gatherstencil.jl:121 */
    STC_ERR_RADIUS = -2,          /* "stencil radius is larger than array axis"  src/array.jl:452, :578 */
    STC_ERR_KERNEL_LENGTH = -3,   /* "Stencil length .. does not match kernel length"  src/stencils/kernel.jl:114-116 */
    STC_ERR_UNSUPPORTED = -4,     /* shape / op / dtype / boundary combination not registered (a MethodError
                                     in the reference, e.g. Use with Conditional padding has no getneighbor) */
    STC_ERR_INVALID = -5,         /* malformed descriptor (null pointer, bad ndims, stride[0] != 1, ...), or a
                                     dest whose element bytes overlap a source's (no defined result) */
    STC_ERR_CUDA = -6,            /* a CUDA runtime call failed */
    STC_ERR_TIMEOUT = -7,         /* a bounded device-side wait ran out; the kernel returned early */
    STC_ERR_NO_DEVICE = -8,       /* no usable sm_100-family GPU */
    STC_ERR_BUDGET = -9,          /* request exceeds the server's HBM budget */
    STC_ERR_BUSY = -10,           /* result not ready / queue full */
    STC_ERR_CANCELLED = -11,      /* job was cancelled before it finished */
    STC_ERR_TOO_LARGE = -12,      /* grid larger than the fixed scratch of stc_life_steps_noalloc */
    STC_ERR_INEXACT = -13,        /* a result does not convert exactly to the destination element type
                                     (the reference's InexactError on setindex!) */
    STC_ERR_BOUNDS = -14          /* debug build (libstencilcuda_debug.so) only: a kernel's computed index
                                     fell outside the buffer it addresses; the access was skipped */
} stc_status;

/* ---- element types ---- */
typedef enum {
    STC_F64 = 0, STC_F32 = 1, STC_BF16 = 2, STC_F16 = 3,
    STC_U8 = 4, STC_BOOL = 5, STC_I32 = 6, STC_I64 = 7
} stc_dtype;

/* ---- registered reductions `f` (the reference takes any Julia function) ----
 * MEAN     Statistics.mean(hood): left fold of `+` over the neighbours in offset order, / L
 * SUM      sum(hood): the same left fold
 * KDOT     kernelproduct(hood): s = 0; s += hood[i] * kernel[i] for i in 1:L   src/stencils/kernel.jl:37-43
 * MIN/MAX  minimum/maximum(hood): left fold of Julia's min/max (NaN-propagating, -0.0 < +0.0)
 * LIFE     outer-totalistic cellular automaton: n = count of nonzero neighbours, c = centre != 0,
 *          result = c ? (survive_mask >> n) & 1 : (birth_mask >> n) & 1   (B3/S23: birth 1<<3,
 *          survive 1<<2 | 1<<3).  Equals the closure `s == 3 || (c && s == 2)` on 0/1 states, which is
 *          what a Bool grid or a 0/1 integer grid holds.  On other states it differs from a closure
 *          over s = sum(hood): the library counts nonzero neighbours (a 2 counts as one live cell),
 *          and results are 0/1.  A caller whose states are not 0/1 must keep the reference path.
 * DIFFUSE  c + alpha * (sum(hood) - L * c): explicit diffusion step, c = centre value.
 */
typedef enum {
    STC_OP_MEAN = 0, STC_OP_SUM = 1, STC_OP_KDOT = 2, STC_OP_MIN = 3, STC_OP_MAX = 4,
    STC_OP_LIFE = 5, STC_OP_DIFFUSE = 6
} stc_opcode;

/* ---- boundary conditions (src/boundary.jl:17-52) and padding (src/padding.jl:28-39) ---- */
typedef enum { STC_REMOVE = 0, STC_WRAP = 1, STC_REFLECT = 2, STC_USE = 3 } stc_boundary;
typedef enum { STC_CONDITIONAL = 0, STC_HALO_IN = 1, STC_HALO_OUT = 2 } stc_padding;

/* ---- stencil shapes with specialised kernels; anything else runs from the offset table ---- */
typedef enum {
    STC_SHAPE_TABLE = 0,       /* arbitrary offsets (Positional, Rectangle, NamedStencil, Annulus, ...) */
    STC_SHAPE_WINDOW = 1, STC_SHAPE_MOORE = 2, STC_SHAPE_VONNEUMANN = 3,
    STC_SHAPE_CIRCLE = 4, STC_SHAPE_CROSS = 5
} stc_shape;

/* A grid: the PARENT array as Julia holds it (for Halo padding this includes the ring of width R).
 * size[d] / stride[d] in elements for d < ndims; stride[0] must be 1. */
typedef struct {
    int32_t ndims;          /* 1..3 */
    int32_t dtype;          /* stc_dtype */
    int64_t size[3];
    int64_t stride[3];
    void*   data;           /* device pointer */
} stc_grid;

/* A stencil: the compile-time offsets Stencils.jl generates, lowered to a table.
 * offsets[k*ndims + d] is component d of offset k (component 0 along the contiguous axis), in
 * the reference's offset order (`offsets`, src/stencil.jl:73-75).  A stencil with fewer dims than the grid keeps
 * the trailing indices fixed (src/stencil.jl:93-95). */
typedef struct {
    int32_t ndims;            /* stencil dims, <= grid ndims */
    int32_t len;              /* L, 1..STC_MAX_LEN */
    int32_t radius;           /* R: the halo width and the radius < axis check (src/array.jl:451-453) */
    int32_t shape;            /* stc_shape; a specialised kernel is used only if the table matches it */
    const int32_t* offsets;   /* host pointer, len*ndims */
    const double*  weights;   /* host pointer, len; KDOT only (else NULL) */
    int32_t weight_dtype;     /* STC_F64 or STC_F32: type of kernel[i] (products are promote(T, W)) */
    int32_t reserved;
} stc_stencil;

#define STC_MAX_LEN 1024
#define STC_MAX_RADIUS 64

typedef struct {
    int32_t  code;            /* stc_opcode */
    int32_t  reserved;
    uint32_t birth_mask;      /* LIFE */
    uint32_t survive_mask;    /* LIFE */
    double   alpha;           /* DIFFUSE */
} stc_op;

typedef struct {
    int32_t boundary;         /* stc_boundary */
    int32_t padding;          /* stc_padding */
    double  padval;           /* Remove(padval) for float grids */
    int64_t padval_int;       /* Remove(padval) for integer / Bool grids */
    int32_t padval_type;      /* Remove: the type of padval, 1 + stc_dtype, or 0 for the grid's own element type
                                 (the reference's default Remove(zero(eltype)), src/array.jl:463).  A padval of
                                 another type promotes the neighbours: they are read as
                                 promote_type(eltype, typeof(padval)) (src/gatherstencil.jl:41-56, :50), so the
                                 fold runs in that type and the result type follows it (stc_neighbor_dtype). */
    int32_t reserved;
} stc_bc;

/* stc_map flags */
/* stc_map_steps flag, BFloat16 / Float16 state only: the precision mode for long runs of 16-bit state.
 * The state is held in memory in the 16-bit type, but between the rounding points it stays Float32.
 * With s = 1..n the steps of this call, P the pass length (8 for BFloat16, 4 for Float16) and
 * m = P * floor((n - 1) / P), the state after step s <= m is rounded to the storage type only when s
 * is a multiple of P: BFloat16 stochastically (round up with probability equal to the distance from the
 * value below; the bits come from a hash of the cell's column-major linear index and s, so results are
 * deterministic), Float16 to nearest.  The last n - m steps (1 to P) run as separate maps, each rounded
 * to nearest.  Results then differ from n maps of
 * 16-bit state (each rounded to nearest); their error against an FP64 run is stated by the benchmark.
 * Runs the temporally blocked 3D path only (3D VonNeumann(1,3) diffusion / mean, Cross(1,3) sum, Wrap
 * or Remove); other runs return STC_ERR_UNSUPPORTED.  Ignored for Float32 / Float64 / integer state. */
#define STC_KEEP_F32 2u
#define STC_ASYNC 1u          /* do not synchronise the stream before returning (errors from the
                                 kernel's own checks surface at the next synchronising call on the
                                 same stream: each stream has its own status slot) */

/* ---- library ---- */
STC_API int         stc_abi_version(void);
STC_API const char* stc_strerror(int status);
STC_API int         stc_last_cuda_error(void);              /* the cudaError_t behind the last STC_ERR_CUDA */
/* 1 in the debug build (device-side bounds tests, STC_ERR_BOUNDS), 0 in the release build. */
STC_API int         stc_debug_bounds(void);
/* Debug build: queue on `stream` a one-thread kernel that reports a failed bounds test through the stream's
 * status slot, as a failing test inside a kernel would (no access is made), so the next synchronising call
 * on that stream returns STC_ERR_BOUNDS.  The release build returns STC_ERR_UNSUPPORTED. */
STC_API int         stc_debug_report_bounds(void* stream);
/* No counterpart in the reference.  Multi-step runs that work on an internal padded pair (3D grids:
 * the temporally blocked path and the edge-patching path) keep that pair's device memory per device
 * for the next run (stream-ordered: a run on another stream waits for the previous one to finish
 * with it).  This frees it on every device, waiting for the device; STC_ERR_BUSY if a run on another
 * host thread holds it at that moment. */
STC_API int         stc_release_workspace(void);

/* Output element type the reference would infer for (op, neighbour dtype, weight dtype)
 * (Base._return_type, src/gatherstencil.jl:41-56), or a negative status. */
STC_API int stc_result_dtype(int32_t opcode, int32_t src_dtype, int32_t weight_dtype);
/* The element type a grid's neighbours are read as: promote_type(src_dtype, typeof(padval)) for Remove
 * with a padval_type (src/gatherstencil.jl:50), else src_dtype; a negative status for a bad padval_type.
 * stc_map writes the result type of that type; stc_map_steps converts each step's result back to the
 * parents' type (STC_ERR_INEXACT where a value does not convert exactly, as the reference's setindex!
 * throws).  The other entry points take grids whose padval needs no promotion (else STC_ERR_UNSUPPORTED). */
STC_API int stc_neighbor_dtype(int32_t src_dtype, const stc_bc* bc);

/* One map: dst[I] = f(stencil(src, I)) for every logical index I.  `src` is the parent array;
 * its logical size is size - 2R per axis for Halo padding.  `dst` is either the logical size
 * (a plain array) or, with dst_padded != 0, a parent of the same padded size whose interior is
 * written (the SwitchingStencilArray case, src/gatherstencil.jl:77-81).  For Halo padding the
 * halo ring of src is refreshed first, as update_boundary! does. */
STC_API int stc_map(const stc_grid* src, const stc_grid* dst, int32_t dst_padded,
            const stc_stencil* stencil, const stc_op* op, const stc_bc* bc,
            void* stream, uint32_t flags);

/* nsteps of `A = mapstencil!(f, A)` on a SwitchingStencilArray whose two parents are a and b,
 * a holding the current source.  On return *out_src_is_b says which parent holds the result
 * (the reference's switch()).  Multi-step runs are temporally blocked where the library has a blocked
 * kernel: Moore(1) cellular automata on packed words (rows of 32 cells or more), 2D Float32 radius-1
 * Window / Moore / VonNeumann maps under Wrap or Remove (runs of 17 steps or more), 3D Float32
 * VonNeumann / Cross radius-1 maps (8 steps or more; 16-bit state in the STC_KEEP_F32 mode); results
 * are those of nsteps separate maps, bit for bit. */
STC_API int stc_map_steps(const stc_grid* a, const stc_grid* b,
                  const stc_stencil* stencil, const stc_op* op, const stc_bc* bc,
                  int64_t nsteps, int32_t* out_src_is_b, void* stream, uint32_t flags);

/* ---- maps over several arrays: mapstencil(f, A, args...) (src/gatherstencil.jl:84-113) ----
 * The reference passes f the stencil of every StencilArray argument at I and the value at I of every
 * plain array (`_getarg`, src/gatherstencil.jl:111-112).  The registered f is a left-to-right sum of
 * one term per argument, t_1 + t_2 + ... + t_n, each term
 *     CENTER  center(hood)            VALUE   arg[I]               (a plain array: stencil/bc NULL)
 *     SUM     sum(neighbors(hood))    MEAN    mean(neighbors(hood))   KDOT  kernelproduct(hood)
 * optionally scaled, alpha * term (scaled != 0), as in `c + 0.1 * sum(neighbors(hood_r))`.  All
 * arithmetic is in the element type of the grids (Float64 or Float32, all the same; alpha is applied
 * in that type); sums fold in offset order exactly as stc_map.  Every StencilArray argument keeps its
 * own stencil, boundary and padding, and Halo arguments get update_boundary! first.  All logical
 * sizes must equal dest's (else STC_ERR_SIZE_MISMATCH, src/gatherstencil.jl:118-124). */
typedef enum {
    STC_TERM_CENTER = 0, STC_TERM_SUM = 1, STC_TERM_MEAN = 2, STC_TERM_KDOT = 3, STC_TERM_VALUE = 4
} stc_term_kind;

typedef struct {
    int32_t kind;                 /* stc_term_kind */
    int32_t scaled;               /* nonzero: alpha * term */
    double  alpha;
    const stc_grid* grid;         /* the argument's parent */
    const stc_stencil* stencil;   /* its stencil (NULL for VALUE) */
    const stc_bc* bc;             /* its boundary and padding (NULL for VALUE) */
} stc_term;

#define STC_MAX_TERMS 4
#define STC_MAX_TERM_LEN 64

/* dest[I] = t_1 + ... + t_n over dest's logical indices; dst_padded as in stc_map, relative to the
 * first term's padding (the SwitchingStencilArray form writes the padded dest parent). */
STC_API int stc_map_terms(const stc_term* terms, int32_t nterms, const stc_grid* dst, int32_t dst_padded,
                          void* stream, uint32_t flags);

/* ---- scatterstencil!(f, op, dest, source) (src/scatterstencil.jl:36-133) ----
 * Each source cell s computes one value per stencil offset k, v_k = f(stencil(source, s))[k], and
 * combines it into dest at s + offset_k: dest[t] = op(dest[t], v_k).  Out-of-range targets are skipped
 * for Remove and Use, wrapped for Wrap and reflected for Reflect (src/scatterstencil.jl:76-112).
 * Registered f: CONST (v_k = constant, as `map(_ -> c, neighbors(hood))`), CENTER
 * (v_k = center(hood)) and WEIGHTED (v_k = center(hood) * kernel[k], a Kernel stencil's weights);
 * registered op: ADD (+), MAX, MIN (Julia's max/min).  2D grids, Float64 or Float32, dest the
 * logical size of source, combined in the element type.  Every dest cell receives its contributions
 * in the order of the reference's pass schedule run on one thread (passes p = 1..2R+1 over the columns
 * j = p, p + 2R + 1, ...; rows in order; offsets in order), so results are deterministic and bit-exact
 * with it (the reference's threaded passes give that order too, except that with Wrap, columns of one
 * pass meet at the seam when the column count is not a multiple of 2R + 1). */
typedef enum { STC_SCATTER_CONST = 0, STC_SCATTER_CENTER = 1, STC_SCATTER_WEIGHTED = 2 } stc_scatter_value;
typedef enum { STC_COMBINE_ADD = 0, STC_COMBINE_MAX = 1, STC_COMBINE_MIN = 2 } stc_combine;

typedef struct {
    int32_t value;       /* stc_scatter_value */
    int32_t combine;     /* stc_combine */
    double  constant;    /* CONST */
} stc_scatter_op;

STC_API int stc_scatter(const stc_grid* src, const stc_grid* dst, const stc_stencil* stencil, const stc_scatter_op* op,
                        const stc_bc* bc, void* stream, uint32_t flags);

/* Host <-> device copies of a grid: `host` is a dense column-major array of the grid's size and type;
 * the device grid may be a strided view, e.g. the interior of a Halo parent (as the reference's
 * StencilArray constructor copies an array into the padded parent, src/padding.jl:102-110, or a user
 * copies a result back with copyto!).  One pitched copy per call (per plane when the planes are not
 * stacked at one pitch; one linear copy when the rows are contiguous); with STC_ASYNC the host buffer must stay valid until the stream reaches the
 * copy (pinned host memory makes the copy asynchronous). */
STC_API int stc_grid_upload(const stc_grid* dst, const void* host, void* stream, uint32_t flags);
STC_API int stc_grid_download(void* host, const stc_grid* src, void* stream, uint32_t flags);

/* update_boundary!: write the halo ring of a Halo-padded parent from its interior. */
STC_API int stc_update_boundary(const stc_grid* parent, int32_t radius, const stc_bc* bc,
                        void* stream, uint32_t flags);

/* FP64 total of the logical grid (Neumaier-compensated; radius/bc.padding locate the interior). */
STC_API int stc_mass(const stc_grid* g, int32_t radius, const stc_bc* bc, double* out_total, void* stream);

/* ---- no-allocation variant of the bit-packed Life path ----
 * No counterpart in the reference.  For callers that cannot allocate device memory: a host whose
 * device memory is all handed out by its own allocator (a Julia CUDA.jl memory pool, a framework's
 * caching allocator, an embedded host that reserved every byte of the device up front), where an
 * allocation by the library would fail or would take memory the owner has already promised
 * elsewhere.  It runs the same bit-packed, temporally blocked Moore(1) kernels as stc_map_steps, but
 * keeps the packed copies in a fixed device array that is part of the library image (4 MiB, held on
 * every GPU that loads the library until the process exits) instead of allocating them.  The caller
 * still owns and passes both parents.  Accepts only what that path runs: a 2D Moore(1) LIFE rule,
 * UInt8/Bool/Int32/Int64 grids whose rows are at least 32 cells and pack into at most 512 words (16384 cells),
 * Wrap or Remove(0), at most 4096*4096 packed cells (larger grids return STC_ERR_TOO_LARGE, other
 * inputs STC_ERR_UNSUPPORTED).  The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for the life of the process; a device reset (cudaDeviceReset)
 * after it is not supported.  All calls share
 * the one array and each call overwrites it: calls whose work overlaps on the GPU (other streams,
 * other host threads) race and must be serialised by the caller.  The call waits for its stream
 * before returning.  Same results and parent switching as stc_map_steps. */
STC_API int stc_life_steps_noalloc(const stc_grid* a, const stc_grid* b, const stc_stencil* stencil,
                                   const stc_op* op, const stc_bc* bc, int64_t nsteps,
                                   int32_t* out_src_is_b, void* stream);

/* ---- tracing: per-launch device time from CUDA events on the launching stream ---- */
/* Enable (1) or disable (0) recording; enabling clears earlier records.  No counterpart in the
 * reference (which has only @time / BenchmarkTools around calls). */
STC_API int stc_profile_enable(int32_t on);
/* JSON object {kernel: {"launches", "ms", "alg_bytes", "updates"}} of everything recorded since
 * enabling; synchronises on the recorded events.  Returns STC_OK, or the buffer size needed (> 0)
 * when `len` is too small. */
STC_API int stc_profile_report(char* buf, size_t len);

/* ---- batched runs: many independent SwitchingStencilArray loops in one launch ---- */
typedef struct stc_batch stc_batch;

STC_API int stc_batch_create(stc_batch** out);
STC_API int stc_batch_destroy(stc_batch* b);
/* Add job: nsteps of stencil/op/bc on grids a (source) and b (scratch).  Returns the job index. */
STC_API int stc_batch_add(stc_batch* b, const stc_grid* a, const stc_grid* bgrid,
                  const stc_stencil* stencil, const stc_op* op, const stc_bc* bc, int64_t nsteps);
/* Choose tile shapes and temporal depth per job (autotune != 0 times candidates on the GPU and
 * caches the winners per (shape, dtype, size class)), build the work list and capture the graph. */
STC_API int stc_batch_plan(stc_batch* b, int32_t autotune, void* stream);
/* Run every job to completion: one graph launch. */
STC_API int stc_batch_run(stc_batch* b, void* stream, uint32_t flags);
/* After run: which parent holds job `idx`'s result. */
STC_API int stc_batch_result(const stc_batch* b, int32_t idx, int32_t* out_src_is_b);
/* Plain reference path for comparison: each job as its own stc_map_steps call. */
STC_API int stc_batch_run_sequential(stc_batch* b, void* stream);

/* ---- serving: continuous batching of stencil jobs with device-resident state ---- */
typedef struct stc_server stc_server;

typedef struct {
    stc_grid    grid;         /* host-side description: data points to HOST memory holding the input,
                                 column-major, rows of size[0] elements stride[1] >= size[0] apart */
    stc_stencil stencil;
    stc_op      op;
    stc_bc      bc;
    int64_t     nsteps;
} stc_job;

/* hbm_fraction: admission budget as a fraction of free device memory (e.g. 0.8);
 * steps_per_tick: most steps any job advances per batched launch (continuous-batching tick). */
STC_API int stc_server_create(stc_server** out, double hbm_fraction, int32_t steps_per_tick);
STC_API int stc_server_destroy(stc_server* s);
/* Queue a job.  Its description and host input are consumed before the call returns (the input is
 * copied straight into the job's device state while the HBM budget allows, else into pinned staging
 * memory), so the caller may reuse the buffer.  Grids of at least 2^21 cells run alone on their own
 * stream (STC_SERVE_SOLO_CELLS overrides the threshold), the others in batched ticks.  *out_id
 * identifies the job. */
STC_API int stc_server_submit(stc_server* s, const stc_job* job, int64_t* out_id);
/* Non-blocking: 1 if the job finished (its result can be fetched), 0 if not, or a status. */
STC_API int stc_server_poll(stc_server* s, int64_t id);
/* A job counts as finished once its result is in pinned host memory (copied from the device as its run
 * ends).  stc_server_fetch copies that result into host memory `out` (logical size, the job's dtype,
 * column-major, dense) and forgets the job; *out_latency_s = submit to result in host memory.  Returns
 * STC_ERR_BUSY if it has not finished. */
STC_API int stc_server_fetch(stc_server* s, int64_t id, void* out, size_t out_bytes,
                     double* out_latency_s);
/* The same without a copy: *out_host receives the pinned buffer holding the result (*out_bytes bytes,
 * column-major, dense); the caller owns it until stc_server_release_buffer returns it to the library's
 * process-wide pool (it may outlive the server). */
STC_API int stc_server_fetch_buffer(stc_server* s, int64_t id, void** out_host, size_t* out_bytes,
                     double* out_latency_s);
STC_API int stc_server_release_buffer(void* host);
/* Completion queue: up to max_ids ids of jobs that finished, failed or were cancelled since the last call
 * (each reported once), waiting up to timeout_s for the first; *n_out = how many were written. */
STC_API int stc_server_ready(stc_server* s, int64_t* ids, int32_t max_ids, double timeout_s, int32_t* n_out);
STC_API int stc_server_cancel(stc_server* s, int64_t id);
/* Block until every submitted job finished or timeout_s passed (STC_ERR_TIMEOUT). */
STC_API int stc_server_drain(stc_server* s, double timeout_s);
/* Counters: jobs admitted, finished, ticks run, peak device bytes held. */
STC_API int stc_server_stats(const stc_server* s, int64_t* admitted, int64_t* finished,
                     int64_t* ticks, int64_t* peak_bytes);

#ifdef __cplusplus
}
#endif
#endif /* STENCIL_CUDA_H */
