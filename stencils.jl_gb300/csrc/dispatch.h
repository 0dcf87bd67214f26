// dispatch.h — host-side registry of compiled map kernels and shared internals of the library.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/stencil_cuda.h"

namespace stc {

struct MapParams;

// Reduction variants a kernel is compiled for (an stc_opcode refined by accumulation type).
enum OpVariant : int {
    OPV_MEAN = 0, OPV_SUM = 1, OPV_KDOT_D = 2, OPV_KDOT_F = 3, OPV_MIN = 4, OPV_MAX = 5,
    OPV_LIFE = 6, OPV_DIFFUSE = 7, OPV_COUNT = 8
};

using LaunchFn = cudaError_t (*)(MapParams& p, cudaStream_t stream, int num_sms);

struct KernelEntry {
    LaunchFn launch = nullptr;       // tiled kernel (TMA or cooperative loads)
    LaunchFn launch_direct = nullptr;  // per-output global gather, for boxes too large for shared memory
    int xt = 1, vs = 1;              // columns per thread, stream slots per thread
    LaunchFn launch_vec = nullptr;   // shape kernels: XV adjacent columns per thread (vector loads)
    int xv = 0, vs_vec = 1;
    int kind = STC_SHAPE_TABLE, R = 0, N = 0;
};

// kind == STC_SHAPE_TABLE for the generic kernels (R, N ignored).  Registering the same key twice
// merges the launchers given (tiled / direct / vector), so each variant registers on its own.
void register_kernel(int src_dtype, int opv, int kind, int R, int N, const KernelEntry& e);
const KernelEntry* find_kernel(int src_dtype, int opv, int kind, int R, int N);

// element size of an stc_dtype (0 if unknown)
int dtype_size(int dt);
bool is_float_dtype(int dt);

// Per-device context: SM count, status word, tensor-map encoder.
struct DeviceCtx {
    int device = -1;
    int num_sms = 0;
    int* status = nullptr;     // device view of a mapped host int, OR-ed by kernels that give up a bounded wait
    int* status_host = nullptr;
    int max_smem_optin = 0;
};
int device_ctx(DeviceCtx** out);

// The status word kernels OR an error bit into (a bounded wait gave up, an inexact conversion) is one of
// a pool of mapped host words, one per stream (or per other key, e.g. a batch whose graph holds the
// device address), so an error of an asynchronous call is reported by the next synchronising call on
// the same stream, not by another caller's.  256 keys per device at a time; beyond that the least
// recently bound key's word is reused.
struct StatusSlot {
    int* dev;
    volatile int* host;
};
StatusSlot status_slot(DeviceCtx* ctx, const void* key);
// reads and clears a slot: STC_OK, or the status its bits stand for
int take_status(const StatusSlot& s);

// remembers the CUDA error behind an STC_ERR_CUDA
int cuda_fail(cudaError_t e);

// The per-device workspace kept between multi-step runs, in stream order on `s`: a buffer of at least
// `bytes`; *cached tells workspace_release whether it is the kept one or a private allocation.
int workspace_acquire(size_t bytes, cudaStream_t s, void** out, bool* cached);
void workspace_release(void* ptr, bool cached, cudaStream_t s);

int validate_map(const stc_grid* src, const stc_grid* dst, int dst_padded, const stc_stencil* st,
                 const stc_op* op, const stc_bc* bc);
// true if the two grids' element byte ranges intersect
bool grids_overlap(const stc_grid* a, const stc_grid* b);
int result_dtype(int op, int sdt, int wdt);
// Julia's promote_type over the library's element types, and the type a grid's neighbours are read as
// (promote_type(eltype, typeof(padval)) for Remove with a padval_type; a negative status if malformed)
int promote_dtype(int a, int b);
int neighbor_dtype(int src, const stc_bc* bc);
// true if the FMA-corrected Float32 quotient by L is exact for every input (checked once per L)
bool fastdiv_f_exact(int L);
// true if `offsets` (len entries of N components) is the table Stencils.jl generates for the shape
bool table_matches_shape(int shape, int R, int N, const int32_t* offsets, int len);
// one map launch (halo fill not included), no synchronisation
int launch_map(const stc_grid* src, const stc_grid* dst, int dst_padded, const stc_stencil* st, const stc_op* op,
               const stc_bc* bc, cudaStream_t stream, DeviceCtx* ctx);

// halo fill (update_boundary!) of a Halo-padded parent
int launch_halo_fill(const stc_grid* parent, int radius, const stc_bc* bc, cudaStream_t stream);

// copy an n[0] x n[1] x n[2] box from src (element offset sorg) to dst (offset dorg), same dtype
int launch_grid_copy(const stc_grid* src, int64_t sorg, const stc_grid* dst, int64_t dorg, const int64_t n[3],
                     cudaStream_t stream);
// the same box converted from src's element type to dst's as Julia's convert does (round to nearest into
// a float type; into an integer or Bool type only exact values, else DEV_ERR_INEXACT in *status)
int launch_grid_convert(const stc_grid* src, int64_t sorg, const stc_grid* dst, int64_t dorg, const int64_t n[3],
                        int* status, cudaStream_t stream);

}  // namespace stc
