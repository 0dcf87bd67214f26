// capi.cu — the extern "C" entry points of libstencilcuda.so for single maps and multi-step runs.
//
// stc_map       replaces gatherstencil!(f, dest, source)            src/gatherstencil.jl:89-103
// stc_map_steps replaces the loop A = gatherstencil!(f, A::Switching) src/gatherstencil.jl:77-83
// stc_update_boundary replaces update_boundary!                      src/array.jl:195-233
// Argument checks return the statuses that mirror the reference's ArgumentErrors.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

#include "dispatch.h"
#include "life.h"
#include "map_kernel.cuh"
#include "profile.h"
#include "tblock.h"

namespace stc {

// ---------------------------------------------------------------------------- registry
static std::map<std::tuple<int, int, int, int, int>, KernelEntry>& registry() {
    static std::map<std::tuple<int, int, int, int, int>, KernelEntry> r;
    return r;
}

void register_kernel(int dt, int opv, int kind, int R, int N, const KernelEntry& e) {
    KernelEntry& x = registry()[std::make_tuple(dt, opv, kind, R, N)];
    if (e.launch) {
        x.launch = e.launch;
        x.xt = e.xt;
        x.vs = e.vs;
    }
    if (e.launch_direct) x.launch_direct = e.launch_direct;
    if (e.launch_vec) {
        x.launch_vec = e.launch_vec;
        x.xv = e.xv;
        x.vs_vec = e.vs_vec;
    }
    x.kind = e.kind;
    x.R = e.R;
    x.N = e.N;
}

const KernelEntry* find_kernel(int dt, int opv, int kind, int R, int N) {
    auto& r = registry();
    auto it = r.find(std::make_tuple(dt, opv, kind, kind == STC_SHAPE_TABLE ? 0 : R, kind == STC_SHAPE_TABLE ? 0 : N));
    return it == r.end() ? nullptr : &it->second;
}

int dtype_size(int dt) {
    switch (dt) {
    case STC_F64: case STC_I64: return 8;
    case STC_F32: case STC_I32: return 4;
    case STC_BF16: case STC_F16: return 2;
    case STC_U8: case STC_BOOL: return 1;
    }
    return 0;
}

bool is_float_dtype(int dt) { return dt == STC_F64 || dt == STC_F32 || dt == STC_BF16 || dt == STC_F16; }

static thread_local int g_last_cuda_error = 0;

int cuda_fail(cudaError_t e) {
    if (e == cudaSuccess) return STC_OK;
    g_last_cuda_error = (int)e;
    return STC_ERR_CUDA;
}

// ---------------------------------------------------------------------------- device context
static std::mutex g_ctx_mu;
static DeviceCtx g_ctx[64];

int device_ctx(DeviceCtx** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { cuda_fail(e); return STC_ERR_NO_DEVICE; }
    if (dev < 0 || dev >= 64) return STC_ERR_NO_DEVICE;
    DeviceCtx& c = g_ctx[dev];
    if (c.device == dev) { *out = &c; return STC_OK; }
    std::lock_guard<std::mutex> g(g_ctx_mu);
    if (c.device != dev) {
        cudaDeviceProp prop;
        e = cudaGetDeviceProperties(&prop, dev);
        if (e != cudaSuccess) return cuda_fail(e);
        if (prop.major < 10) return STC_ERR_NO_DEVICE;
        c.num_sms = prop.multiProcessorCount;
        c.max_smem_optin = (int)prop.sharedMemPerBlockOptin;
        int* h = nullptr;
        e = cudaHostAlloc((void**)&h, sizeof(int), cudaHostAllocMapped);
        if (e != cudaSuccess) return cuda_fail(e);
        *h = 0;
        int* d = nullptr;
        e = cudaHostGetDevicePointer((void**)&d, h, 0);
        if (e != cudaSuccess) return cuda_fail(e);
        c.status = d;
        c.status_host = h;
        // The runs' stream-ordered scratch (packed Life grids and exchange slots, padded pairs, batch
        // scratch) goes back to the device's default pool, which by default unmaps it at every
        // synchronisation, so a synchronising caller paid for fresh pages on every call.  Keep up to 1 GiB
        // mapped (a higher threshold set by the application stays).
        cudaMemPool_t pool;
        if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
            uint64_t cur = 0, keep = 1ull << 30;
            if (cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &cur) == cudaSuccess && cur < keep)
                cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
        }
        cudaGetLastError();
        c.device = dev;
    }
    *out = &c;
    return STC_OK;
}

// ---------------------------------------------------------------------------- workspace
// The internal padded pair of a multi-step run is large (two grids plus their rings), and mapping fresh
// pages for it on every call costs as much as tens of steps.  Each device keeps the last one; a call
// takes it in stream order (waiting on the event the previous user recorded) and gives it back with an
// event on its own stream, so calls on different streams never overlap on it.  A call that finds it
// taken by another host thread gets a private stream-ordered allocation instead.
struct Workspace {
    void* ptr = nullptr;
    size_t bytes = 0;
    cudaEvent_t done = nullptr;
    bool busy = false;
};
static std::mutex g_ws_mu;
static Workspace g_ws[64];

int workspace_acquire(size_t bytes, cudaStream_t s, void** out, bool* cached) {
    *out = nullptr;
    *cached = false;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess || dev < 0 || dev >= 64) return STC_ERR_NO_DEVICE;
    {
        std::lock_guard<std::mutex> g(g_ws_mu);
        Workspace& w = g_ws[dev];
        if (!w.busy) {
            if (w.bytes < bytes) {
                if (w.ptr) {
                    cudaFree(w.ptr);   // waits for the device: no earlier user still reads it
                    w.ptr = nullptr;
                    w.bytes = 0;
                }
                if (cudaMalloc(&w.ptr, bytes) != cudaSuccess) {
                    cudaGetLastError();
                    w.ptr = nullptr;
                    return STC_ERR_CUDA;
                }
                w.bytes = bytes;
            } else if (w.done) {
                if ((e = cudaStreamWaitEvent(s, w.done, 0)) != cudaSuccess) return cuda_fail(e);
            }
            if (!w.done && (e = cudaEventCreateWithFlags(&w.done, cudaEventDisableTiming)) != cudaSuccess)
                return cuda_fail(e);
            w.busy = true;
            *out = w.ptr;
            *cached = true;
            return STC_OK;
        }
    }
    if ((e = cudaMallocAsync(out, bytes, s)) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return STC_ERR_CUDA;
    }
    return STC_OK;
}

void workspace_release(void* ptr, bool cached, cudaStream_t s) {
    if (!ptr) return;
    if (!cached) {
        cudaFreeAsync(ptr, s);
        return;
    }
    int dev = 0;
    cudaGetDevice(&dev);
    std::lock_guard<std::mutex> g(g_ws_mu);
    Workspace& w = g_ws[dev];
    cudaEventRecord(w.done, s);
    w.busy = false;
}

// ---------------------------------------------------------------------------- status slots
constexpr int kStatusSlots = 256;
struct SlotPool {
    int* host = nullptr;
    int* dev = nullptr;
    std::map<const void*, std::pair<int, uint64_t>> bound;   // key -> (slot, last use)
    uint64_t clock = 0;
};
static SlotPool g_slots[64];

StatusSlot status_slot(DeviceCtx* ctx, const void* key) {
    std::lock_guard<std::mutex> g(g_ctx_mu);
    SlotPool& P = g_slots[ctx->device];
    if (!P.host) {
        int* h = nullptr;
        int* d = nullptr;
        if (cudaHostAlloc((void**)&h, sizeof(int) * kStatusSlots, cudaHostAllocMapped) == cudaSuccess &&
            cudaHostGetDevicePointer((void**)&d, h, 0) == cudaSuccess) {
            memset(h, 0, sizeof(int) * kStatusSlots);
            P.host = h;
            P.dev = d;
        } else {
            cudaGetLastError();   // no pool: every key shares the context's own word
            return StatusSlot{ctx->status, ctx->status_host};
        }
    }
    ++P.clock;
    auto it = P.bound.find(key);
    if (it != P.bound.end()) {
        it->second.second = P.clock;
        return StatusSlot{P.dev + it->second.first, P.host + it->second.first};
    }
    int slot = (int)P.bound.size();
    if (slot >= kStatusSlots) {
        auto lru = P.bound.begin();
        for (auto j = P.bound.begin(); j != P.bound.end(); ++j)
            if (j->second.second < lru->second.second) lru = j;
        slot = lru->second.first;
        P.bound.erase(lru);
    }
    P.bound[key] = {slot, P.clock};
    return StatusSlot{P.dev + slot, P.host + slot};
}

int take_status(const StatusSlot& sl) {
    const int v = *sl.host;
    if (!v) return STC_OK;
    *sl.host = 0;
    if (v & DEV_ERR_TIMEOUT) return STC_ERR_TIMEOUT;
    if (v & DEV_ERR_BOUNDS) return STC_ERR_BOUNDS;
    return STC_ERR_INEXACT;
}

// waits for the stream, then reads and clears its status slot
static int finish_sync(cudaStream_t s, DeviceCtx* ctx) {
    cudaError_t e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return cuda_fail(e);
    return take_status(status_slot(ctx, s));
}

// ---------------------------------------------------------------------------- type promotion
// Julia's promote_type over the element types the library takes: Bool gives way to anything; an
// integer and a float give the float; integers the wider (UInt8 < Int32 < Int64); floats the wider, with
// BFloat16 and Float16 meeting at Float32 (BFloat16s.jl's promote_rule).
int promote_dtype(int a, int b) {
    if (a == b) return a;
    if (a == STC_BOOL) return b;
    if (b == STC_BOOL) return a;
    const bool fa = is_float_dtype(a), fb = is_float_dtype(b);
    if (fa != fb) return fa ? a : b;
    if (!fa) {
        auto rank = [](int d) { return d == STC_U8 ? 1 : d == STC_I32 ? 2 : 3; };
        return rank(a) >= rank(b) ? a : b;
    }
    if (a == STC_F64 || b == STC_F64) return STC_F64;
    return STC_F32;   // F32 with a 16-bit type, or BFloat16 with Float16
}

int neighbor_dtype(int src, const stc_bc* bc) {
    if (!bc || bc->boundary != STC_REMOVE || bc->padval_type == 0) return src;
    const int pt = bc->padval_type - 1;
    if (pt < 0 || dtype_size(pt) == 0) return STC_ERR_INVALID;
    return promote_dtype(src, pt);
}

// ---------------------------------------------------------------------------- tensor maps
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                  const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encoder() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiledFn)p;
    });
    return fn;
}

static CUtensorMapDataType tma_dtype(int dt) {
    switch (dt) {
    case STC_F64: return CU_TENSOR_MAP_DATA_TYPE_FLOAT64;
    case STC_F32: return CU_TENSOR_MAP_DATA_TYPE_FLOAT32;
    case STC_BF16: return CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
    case STC_F16: return CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
    case STC_I32: return CU_TENSOR_MAP_DATA_TYPE_INT32;
    case STC_I64: return CU_TENSOR_MAP_DATA_TYPE_INT64;
    default: return CU_TENSOR_MAP_DATA_TYPE_UINT8;
    }
}

// ---------------------------------------------------------------------------- validation
int result_dtype(int op, int sdt, int wdt) {
    const bool sf = is_float_dtype(sdt);
    if (dtype_size(sdt) == 0) return STC_ERR_UNSUPPORTED;
    switch (op) {
    case STC_OP_MEAN: return sf ? sdt : STC_F64;
    case STC_OP_SUM: return sf ? sdt : (sdt == STC_BOOL ? STC_I64 : sdt);
    case STC_OP_KDOT:
        if (sf && sdt != STC_F64 && wdt == STC_F32) return sdt;
        return STC_F64;
    case STC_OP_MIN: case STC_OP_MAX: return sdt;
    case STC_OP_LIFE: return sf ? STC_ERR_UNSUPPORTED : sdt;
    case STC_OP_DIFFUSE: return sf ? sdt : STC_ERR_UNSUPPORTED;
    }
    return STC_ERR_UNSUPPORTED;
}

static int op_variant(const stc_op* op, int sdt, int wdt) {
    switch (op->code) {
    case STC_OP_MEAN: return OPV_MEAN;
    case STC_OP_SUM: return OPV_SUM;
    case STC_OP_KDOT: return (is_float_dtype(sdt) && sdt != STC_F64 && wdt == STC_F32) ? OPV_KDOT_F : OPV_KDOT_D;
    case STC_OP_MIN: return OPV_MIN;
    case STC_OP_MAX: return OPV_MAX;
    case STC_OP_LIFE: return OPV_LIFE;
    case STC_OP_DIFFUSE: return OPV_DIFFUSE;
    }
    return -1;
}

static int check_grid(const stc_grid* g) {
    if (!g || g->ndims < 1 || g->ndims > 3 || dtype_size(g->dtype) == 0) return STC_ERR_INVALID;
    if (g->size[0] > 1 && g->stride[0] != 1) return STC_ERR_INVALID;
    for (int d = 0; d < g->ndims; ++d)
        if (g->size[d] < 0 || g->stride[d] < 0) return STC_ERR_INVALID;
    return STC_OK;
}

// True if the byte ranges spanned by a's and b's elements intersect (conservative for interleaved
// views of one buffer).  A dest that shares memory with its source has no defined result: the tiled
// kernels read boxes other CTAs are writing, and the reference's threads race the same way.
bool grids_overlap(const stc_grid* a, const stc_grid* b) {
    auto span = [](const stc_grid* g, uintptr_t& lo, uintptr_t& hi) {
        int64_t last = 0;
        for (int d = 0; d < g->ndims; ++d) {
            if (g->size[d] == 0) return false;
            last += (g->size[d] - 1) * g->stride[d];
        }
        lo = (uintptr_t)g->data;
        hi = lo + (uintptr_t)((last + 1) * (int64_t)dtype_size(g->dtype));
        return true;
    };
    uintptr_t al, ah, bl, bh;
    if (!span(a, al, ah) || !span(b, bl, bh)) return false;
    return al < bh && bl < ah;
}

int validate_map(const stc_grid* src, const stc_grid* dst, int dst_padded, const stc_stencil* st,
                 const stc_op* op, const stc_bc* bc) {
    int rc;
    if ((rc = check_grid(src)) || (rc = check_grid(dst))) return rc;
    if (!st || !op || !bc || !st->offsets) return STC_ERR_INVALID;
    if (st->len < 1 || st->len > STC_MAX_LEN || st->ndims < 1 || st->ndims > src->ndims) return STC_ERR_INVALID;
    if (st->radius < 0 || st->radius > STC_MAX_RADIUS) return STC_ERR_UNSUPPORTED;
    for (int k = 0; k < st->len * st->ndims; ++k)
        if (st->offsets[k] > st->radius || st->offsets[k] < -st->radius) return STC_ERR_UNSUPPORTED;
    if (op->code == STC_OP_KDOT && !st->weights) return STC_ERR_KERNEL_LENGTH;
    if (op->code == STC_OP_LIFE && st->len > 31) return STC_ERR_UNSUPPORTED;
    if (bc->boundary < STC_REMOVE || bc->boundary > STC_USE) return STC_ERR_INVALID;
    if (bc->padding < STC_CONDITIONAL || bc->padding > STC_HALO_OUT) return STC_ERR_INVALID;
    if (bc->boundary == STC_USE && bc->padding == STC_CONDITIONAL) return STC_ERR_UNSUPPORTED;
    const int ndt = neighbor_dtype(src->dtype, bc);
    if (ndt < 0) return ndt;
    const int rdt = result_dtype(op->code, ndt, st->weight_dtype);
    if (rdt < 0) return rdt;
    if (dst->dtype != rdt) return STC_ERR_UNSUPPORTED;
    if (dst->ndims != src->ndims) return STC_ERR_SIZE_MISMATCH;
    // StencilArray constructor: radius < each parent axis (src/array.jl:451-453)
    for (int d = 0; d < src->ndims; ++d)
        if (!(st->radius < src->size[d])) return STC_ERR_RADIUS;
    const bool halo = bc->padding != STC_CONDITIONAL;
    for (int d = 0; d < src->ndims; ++d) {
        const int64_t logical = src->size[d] - (halo ? 2 * st->radius : 0);
        if (logical < 0) return STC_ERR_RADIUS;
        const int64_t want = logical + ((halo && dst_padded) ? 2 * st->radius : 0);
        if (dst->size[d] != want) return STC_ERR_SIZE_MISMATCH;  // _checksizes (src/gatherstencil.jl:118-124)
    }
    for (const stc_grid* g : {src, dst}) {
        int64_t cells = 1;
        for (int d = 0; d < g->ndims; ++d) cells *= g->size[d];
        if (cells && !g->data) return STC_ERR_INVALID;
    }
    return STC_OK;
}

// ---------------------------------------------------------------------------- shapes
static void generate_shape(int kind, int R, int N, std::vector<int>& out) {
    out.clear();
    const int zr = N >= 3 ? R : 0, yr = N >= 2 ? R : 0;
    for (int z = -zr; z <= zr; ++z)
        for (int y = -yr; y <= yr; ++y)
            for (int x = -R; x <= R; ++x) {
                const int m = abs(x) + abs(y) + abs(z);
                const int s2 = x * x + y * y + z * z;
                const int zeros = (x == 0) + (N >= 2 && y == 0) + (N >= 3 && z == 0);
                bool in = false;
                if (kind == STC_SHAPE_WINDOW) in = N <= 2;
                else if (kind == STC_SHAPE_MOORE) in = m != 0;
                else if (kind == STC_SHAPE_VONNEUMANN) in = m >= 1 && m <= R;
                else if (kind == STC_SHAPE_CIRCLE) in = s2 <= R * R + R;
                else if (kind == STC_SHAPE_CROSS) in = zeros >= N - 1;
                if (!in) continue;
                out.push_back(x);
                if (N >= 2) out.push_back(y);
                if (N >= 3) out.push_back(z);
            }
}

bool table_matches_shape(int shape, int R, int N, const int32_t* offsets, int len) {
    if (shape == STC_SHAPE_TABLE) return false;
    std::vector<int> t;
    generate_shape(shape, R, N, t);
    if ((int)t.size() != len * N) return false;
    return std::memcmp(t.data(), offsets, t.size() * sizeof(int)) == 0;
}

static bool table_is_shape(const stc_stencil* st, int grid_ndims) {
    if (st->ndims != grid_ndims) return false;
    return table_matches_shape(st->shape, st->radius, st->ndims, st->offsets, st->len);
}

// ---------------------------------------------------------------------------- exact division by L
// The Float32 quotient path q' = RN(q + RN(a - q*L)*r), q = RN(a*r), r = RN(1/L) is used for a given L
// only if it equals the correctly rounded a / L for every mantissa of the binade [1, 2): the kernels'
// guard keeps intermediates normal, where the pattern repeats in every binade.  The reference quotient
// is computed in double and rounded once more to float, which is exact for division (53 >= 2*24+2).
bool fastdiv_f_exact(int L) {
    static std::mutex mu;
    static std::map<int, bool> cache;
    std::lock_guard<std::mutex> g(mu);
    auto it = cache.find(L);
    if (it != cache.end()) return it->second;
    const float r = (float)(1.0 / (double)L);
    const float fl = (float)L;
    bool ok = L > 0;
    for (uint32_t m = 0; ok && m < (1u << 23); ++m) {
        const uint32_t bits = 0x3f800000u | m;
        float a;
        std::memcpy(&a, &bits, 4);
        volatile float q = a * r;
        const float e = std::fmaf(-q, fl, a);
        const float q2 = std::fmaf(e, r, q);
        const float want = (float)((double)a / (double)L);
        uint32_t u1, u2;
        std::memcpy(&u1, &q2, 4);
        std::memcpy(&u2, &want, 4);
        ok = u1 == u2;
    }
    cache[L] = ok;
    return ok;
}

// ---------------------------------------------------------------------------- planning
static inline int64_t cdiv(int64_t a, int64_t b) { return (a + b - 1) / b; }
static inline int64_t align_up(int64_t a, int64_t b) { return cdiv(a, b) * b; }

// Fills MapParams for one map of src -> dst and launches it (no synchronisation).
int launch_map(const stc_grid* src, const stc_grid* dst, int dst_padded, const stc_stencil* st, const stc_op* op,
               const stc_bc* bc, cudaStream_t stream, DeviceCtx* ctx) {
    static thread_local MapParams* pp = nullptr;
    if (!pp) {
        void* mem = nullptr;
        if (posix_memalign(&mem, alignof(MapParams), sizeof(MapParams))) return STC_ERR_INVALID;
        pp = (MapParams*)mem;
    }
    MapParams& p = *pp;
    memset(&p, 0, sizeof(MapParams));
    const int nd = src->ndims;
    const int es = dtype_size(src->dtype);
    const bool halo = bc->padding != STC_CONDITIONAL;
    const int R = st->radius;
    p.src = src->data;
    p.dst = dst->data;
    p.ndims = nd;
    p.halo = halo;
    p.boundary = bc->boundary;
    p.status = status_slot(ctx, stream).dev;
    p.L = st->len;
    p.rcp_f = (float)(1.0 / (double)st->len);
    p.Lf = (float)st->len;
    p.Ld = (double)st->len;
    p.alpha_f = (float)op->alpha;
    p.fastdiv_f = (op->code == STC_OP_MEAN && !is_float_dtype(src->dtype)) ? 0
                  : (op->code == STC_OP_MEAN && src->dtype != STC_F64) ? (int)fastdiv_f_exact(st->len) : 0;
    p.birth = op->birth_mask;
    p.survive = op->survive_mask;
    p.alpha = op->alpha;
    int64_t cells = 1;
    for (int d = 0; d < 3; ++d) {
        p.n[d] = d < nd ? src->size[d] - (halo ? 2 * R : 0) : 1;
        p.sst[d] = d < nd ? src->stride[d] : 0;
        p.dstr[d] = d < nd ? dst->stride[d] : 0;
        p.hx[d] = (d < nd && halo) ? R : 0;
        p.src_org += (int64_t)p.hx[d] * p.sst[d];
        if (halo && dst_padded && d < nd) p.dst_org += (int64_t)R * p.dstr[d];
        cells *= p.n[d];
    }
    if (cells == 0) return STC_OK;
    // A Halo parent whose base is not 16-byte aligned (its ring starts just before an aligned interior)
    // gets its tensor map from the 16-byte boundary below the base: the extra leading columns are memory
    // of the same allocation and only ever land in the box's unused left padding.  (Not for Conditional
    // grids, whose x < 0 cells must read as TMA's zero fill.)
    const int es_src = dtype_size(src->dtype);
    int tma_shift = 0;
    if (halo && ((uintptr_t)src->data % 16) != 0 && ((uintptr_t)src->data % es_src) == 0)
        tma_shift = (int)(((uintptr_t)src->data % 16) / es_src);
    p.hx[0] += tma_shift;   // from here on hx[0] is the tensor-map coordinate of logical x = 0
    // Remove's padval in the source element type
    p.padi = bc->padval_int;
    p.padf = bc->padval;
    if (!is_float_dtype(src->dtype)) p.padf = (double)bc->padval_int;
    // offsets (padded with zeros for trailing grid axes) and weights
    int rmax[3] = {0, 0, 0};
    for (int k = 0; k < st->len; ++k)
        for (int d = 0; d < 3; ++d) {
            const int o = d < st->ndims ? st->offsets[k * st->ndims + d] : 0;
            p.off[k][d] = (int8_t)o;
            rmax[d] = std::max(rmax[d], abs(o));
        }
    if (st->weights)
        for (int k = 0; k < st->len; ++k) {
            p.w[k] = st->weights[k];
            p.wf[k] = (float)st->weights[k];
        }
    p.rx = rmax[0];
    p.ry = rmax[1];
    p.rz = rmax[2];

    const int opv = op_variant(op, src->dtype, st->weight_dtype);
    const KernelEntry* e = nullptr;
    if (table_is_shape(st, nd)) e = find_kernel(src->dtype, opv, st->shape, R, st->ndims);
    if (e && !(p.rx == R && p.ry == (nd >= 2 ? R : 0) && p.rz == (nd >= 3 ? R : 0))) e = nullptr;
    if (!e) e = find_kernel(src->dtype, opv, STC_SHAPE_TABLE, 0, 0);
    if (!e) return STC_ERR_UNSUPPORTED;

    // tile geometry
    const bool specialised = e->kind != STC_SHAPE_TABLE;
    // The vector-column variant needs the tile's first column on an XV-aligned shared-memory index.
    // padl (below) is congruent to the tensor-map x of logical 0 modulo 16 bytes, so that is hx[0] % XV.
    const char* nv = getenv("STC_NO_VEC");   // tuning / test override: one column per lane
    const bool vec = specialised && e->launch_vec && !(nv && nv[0] == '1') && (p.hx[0] % e->xv) == 0;
    const int xcols = vec ? e->xv : e->xt, vslots = vec ? e->vs_vec : e->vs;
    p.tiles3d = specialised ? (e->N == 3) : (nd == 3);
    p.tw = 32 * xcols;
    p.th = p.tiles3d ? kMapWarps : kMapWarps * vslots;
    p.tz = p.tiles3d ? vslots : 1;
    const int V = 16 / es;
    p.padl = p.rx + (int)(((p.hx[0] - p.rx) % V + V) % V);
    const int reach = vec ? (int)align_up(p.rx, e->xv) : p.rx;   // loaded columns right of the tile
    p.bw = (int)align_up(p.padl + p.tw + reach, V);
    p.bh = p.th + 2 * p.ry;
    p.bd = p.tz + 2 * p.rz;
    p.ntx = cdiv(p.n[0], p.tw);
    p.nty = cdiv(p.n[1], p.th);
    p.ntz = cdiv(p.n[2], p.tz);
    p.ntiles = p.ntx * p.nty * p.ntz;
    p.box_bytes = (uint32_t)((int64_t)p.bw * p.bh * p.bd * es);
    p.stage_bytes = (uint32_t)align_up(p.box_bytes, 128);
    const int64_t smem_cap = (int64_t)ctx->max_smem_optin - 1024 - 8 * kMaxStages;

    char* tma_base = (char*)src->data - (size_t)tma_shift * es;
    bool tma = nd >= 2 && encoder() != nullptr && ((uintptr_t)tma_base % 16 == 0) && p.bw <= 256 &&
               p.bh <= 256 && p.bd <= 256 && 2 * (int64_t)p.stage_bytes <= smem_cap;
    for (int d = 1; d < nd; ++d)
        if ((src->stride[d] * es) % 16 != 0) tma = false;
    // TMA box coordinates are signed 32-bit: axes this long take the cooperative (64-bit) loader
    for (int d = 0; d < nd; ++d)
        if (src->size[d] + tma_shift + 512 >= (1ll << 31)) tma = false;
    if (tma) {
        p.stages = (int)std::min<int64_t>(kMaxStages, std::max<int64_t>(2, (64 * 1024) / p.stage_bytes));
        while ((int64_t)p.stages * p.stage_bytes > smem_cap) --p.stages;
        cuuint64_t gdim[3], gstr[2];
        cuuint32_t box[3] = {(cuuint32_t)p.bw, (cuuint32_t)p.bh, (cuuint32_t)p.bd}, est[3] = {1, 1, 1};
        for (int d = 0; d < nd; ++d) gdim[d] = (cuuint64_t)src->size[d] + (d == 0 ? tma_shift : 0);
        for (int d = 1; d < nd; ++d) gstr[d - 1] = (cuuint64_t)(src->stride[d] * es);
        CUresult r = encoder()(&p.tmap, tma_dtype(src->dtype), (cuuint32_t)nd, tma_base, gdim, gstr, box, est,
                               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                               CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) tma = false;
    }
    p.use_tma = tma;
    if (!tma) p.stages = 1;
    // After a TMA copy, out-of-range cells hold zeros: right for Halo (never read) and Remove(0).
    bool zero_pad = bc->boundary == STC_REMOVE &&
                    (is_float_dtype(src->dtype) ? (bc->padval == 0.0 && !std::signbit(bc->padval)) : bc->padval_int == 0);
    p.fixup = !halo && !zero_pad;

    cudaError_t err;
    void* prof = prof_begin(stream);
    const char* kname;
    if (!tma && (int64_t)p.stage_bytes > smem_cap) {
        if (!e->launch_direct) e = find_kernel(src->dtype, opv, STC_SHAPE_TABLE, 0, 0);
        if (!e || !e->launch_direct) return STC_ERR_UNSUPPORTED;
        err = e->launch_direct(p, stream, ctx->num_sms);
        kname = "map_direct";
    } else {
        err = (vec ? e->launch_vec : e->launch)(p, stream, ctx->num_sms);
        kname = vec ? (tma ? "map_vec_tma" : "map_vec_ldg")
                    : specialised ? (tma ? "map_shape_tma" : "map_shape_ldg") : (tma ? "map_table_tma" : "map_table_ldg");
    }
    prof_end(prof, stream, kname, (double)cells * (es + dtype_size(dst->dtype)), (double)cells);
    return cuda_fail(err);
}

#ifdef STC_DEBUG_BOUNDS
__global__ void report_bounds_kernel(int* status) { atomicOr(status, DEV_ERR_BOUNDS); }
#endif

}  // namespace stc

using namespace stc;

extern "C" {

int stc_abi_version(void) { return STC_ABI_VERSION; }

int stc_debug_bounds(void) {
#ifdef STC_DEBUG_BOUNDS
    return 1;
#else
    return 0;
#endif
}

int stc_debug_report_bounds(void* stream) {
#ifdef STC_DEBUG_BOUNDS
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    report_bounds_kernel<<<1, 1, 0, s>>>(status_slot(ctx, s).dev);
    return cuda_fail(cudaGetLastError());
#else
    (void)stream;
    return STC_ERR_UNSUPPORTED;
#endif
}

const char* stc_strerror(int status) {
    switch (status) {
    case STC_OK: return "ok";
    case STC_ERR_SIZE_MISMATCH: return "Source array sizes must match";
    case STC_ERR_RADIUS: return "stencil radius is larger than array axis";
    case STC_ERR_KERNEL_LENGTH: return "Stencil length does not match kernel length";
    case STC_ERR_UNSUPPORTED: return "unsupported shape / op / dtype / boundary combination";
    case STC_ERR_INVALID: return "invalid argument";
    case STC_ERR_CUDA: return "CUDA error";
    case STC_ERR_TIMEOUT: return "a bounded device wait timed out";
    case STC_ERR_NO_DEVICE: return "no sm_100-family GPU";
    case STC_ERR_BUDGET: return "request exceeds the HBM budget";
    case STC_ERR_BUSY: return "not finished";
    case STC_ERR_CANCELLED: return "cancelled";
    case STC_ERR_TOO_LARGE: return "grid exceeds the fixed no-allocation scratch (4096*4096 cells)";
    case STC_ERR_INEXACT: return "InexactError: a result does not convert exactly to the destination element type";
    case STC_ERR_BOUNDS: return "a device-side bounds test failed (debug build); the access was skipped";
    }
    return "unknown status";
}

int stc_last_cuda_error(void) { return g_last_cuda_error; }

int stc_release_workspace(void) {
    int cur = 0;
    if (cudaGetDevice(&cur) != cudaSuccess) return STC_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> g(g_ws_mu);
    int rc = STC_OK;
    for (int d = 0; d < 64; ++d) {
        Workspace& w = g_ws[d];
        if (!w.ptr && !w.done) continue;
        if (w.busy) { rc = STC_ERR_BUSY; continue; }
        cudaSetDevice(d);
        if (w.ptr) cudaFree(w.ptr);   // waits for the device
        if (w.done) cudaEventDestroy(w.done);
        w = Workspace{};
    }
    cudaSetDevice(cur);
    return rc;
}

int stc_result_dtype(int32_t opcode, int32_t src_dtype, int32_t weight_dtype) {
    return result_dtype(opcode, src_dtype, weight_dtype);
}

int stc_neighbor_dtype(int32_t src_dtype, const stc_bc* bc) {
    if (dtype_size(src_dtype) == 0) return STC_ERR_INVALID;
    return neighbor_dtype(src_dtype, bc);
}

}  // extern "C"

namespace stc {
// A dense device grid of `dt` with g's sizes, in stream-ordered memory (freed with cudaFreeAsync).
static int dense_like(const stc_grid* g, int dt, stc_grid* out, cudaStream_t s) {
    *out = *g;
    out->dtype = dt;
    int64_t cells = 1;
    for (int d = 0; d < 3; ++d) {
        const int64_t n = d < g->ndims ? g->size[d] : 1;
        out->stride[d] = d < g->ndims ? cells : 0;
        cells *= n;
    }
    out->data = nullptr;
    cudaError_t e = cudaMallocAsync(&out->data, (size_t)std::max<int64_t>(cells, 1) * dtype_size(dt), s);
    return cuda_fail(e);
}

static void sizes3(const stc_grid* g, int64_t n[3]) {
    for (int d = 0; d < 3; ++d) n[d] = d < g->ndims ? g->size[d] : 1;
}

// stc_map with a padval of another type: the source parent (ring included) is converted to the
// neighbour type promote_type(eltype, typeof(padval)) (src/gatherstencil.jl:50) and mapped from there.
static int map_promoted(const stc_grid* src, const stc_grid* dst, int dst_padded, const stc_stencil* st,
                        const stc_op* op, const stc_bc* bc, int ndt, cudaStream_t s, DeviceCtx* ctx) {
    stc_grid t;
    int rc = dense_like(src, ndt, &t, s);
    if (rc) return rc;
    int64_t n[3];
    sizes3(src, n);
    stc_bc b2 = *bc;
    b2.padval_type = 0;
    rc = launch_grid_convert(src, 0, &t, 0, n, status_slot(ctx, s).dev, s);
    if (!rc) rc = launch_halo_fill(&t, st->radius, &b2, s);
    if (!rc) rc = launch_map(&t, dst, dst_padded, st, op, &b2, s, ctx);
    cudaFreeAsync(t.data, s);
    return rc;
}
}  // namespace stc

extern "C" {

int stc_map(const stc_grid* src, const stc_grid* dst, int32_t dst_padded, const stc_stencil* st, const stc_op* op,
            const stc_bc* bc, void* stream, uint32_t flags) {
    int rc = validate_map(src, dst, dst_padded, st, op, bc);
    if (rc) return rc;
    if (grids_overlap(src, dst)) return STC_ERR_INVALID;
    DeviceCtx* ctx = nullptr;
    if ((rc = device_ctx(&ctx))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int ndt = neighbor_dtype(src->dtype, bc);
    if (ndt != src->dtype) {
        if ((rc = map_promoted(src, dst, dst_padded, st, op, bc, ndt, s, ctx))) return rc;
        return (flags & STC_ASYNC) ? STC_OK : finish_sync(s, ctx);
    }
    if ((rc = launch_halo_fill(src, st->radius, bc, s))) return rc;
    if ((rc = launch_map(src, dst, dst_padded, st, op, bc, s, ctx))) return rc;
    if (!(flags & STC_ASYNC)) rc = finish_sync(s, ctx);
    return rc;
}

}  // extern "C"

namespace stc {
// Wrap, Reflect or nonzero Remove on a Conditional 3D SwitchingStencilArray: the steps run on an
// internal Halo-padded pair whose ring is refreshed (K2) before every step, so every tile's input box
// arrives whole from TMA and no edge tile needs patching.  The ring holds exactly the values the
// Conditional rules give (bounded_index / padval), so each step is bit-identical to the direct one.
// Afterwards state n goes to the parent the reference leaves it in and state n-1 to the other.
// Returns STC_OK with *done = 0 when it does not apply or scratch memory is not available.
static int padded_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op,
                        const stc_bc* bc, int64_t nsteps, int* src_is_b, cudaStream_t s, DeviceCtx* ctx,
                        int64_t* done) {
    *done = 0;
    if (nsteps < 4 || a->ndims != 3 || bc->padding != STC_CONDITIONAL || bc->boundary == STC_USE) return STC_OK;
    if (const char* e = getenv("STC_NO_PADDED")) if (e[0] == '1') return STC_OK;   // tuning / test override
    const bool zero_pad = bc->boundary == STC_REMOVE &&
                          (is_float_dtype(a->dtype) ? (bc->padval == 0.0 && !std::signbit(bc->padval)) : bc->padval_int == 0);
    if (zero_pad) return STC_OK;   // TMA's zero fill already gives Remove(0) without patching
    const int R = st->radius;
    const int es = dtype_size(a->dtype);
    int64_t P[3], n[3];
    for (int d = 0; d < 3; ++d) {
        n[d] = a->size[d];
        P[d] = n[d] + 2 * R;
    }
    // Rows: `lead` unused cells, the R ring cells, the interior, the R ring cells, padding; lead + R is a
    // multiple of 128 bytes and so is the pitch, so every interior row starts on a 128-byte line (the
    // map's row stores stay whole lines).
    const int64_t line = 128 / es;
    const int64_t lead = (R + line - 1) / line * line - R;
    const int64_t pitch = (lead + P[0] + line - 1) / line * line;
    const size_t cells = (size_t)pitch * P[1] * P[2];
    void* mem = nullptr;
    bool cached = false;
    if (workspace_acquire(2 * cells * es, s, &mem, &cached) != STC_OK) return STC_OK;
    stc_grid pg[2];
    for (int i = 0; i < 2; ++i) {
        pg[i].ndims = 3;
        pg[i].dtype = a->dtype;
        for (int d = 0; d < 3; ++d) pg[i].size[d] = P[d];
        pg[i].stride[0] = 1;
        pg[i].stride[1] = pitch;
        pg[i].stride[2] = pitch * P[1];
        pg[i].data = (char*)mem + (i * cells + lead) * es;
    }
    stc_bc hb = *bc;
    hb.padding = STC_HALO_OUT;
    const int64_t inner = R + R * pitch + R * pitch * P[1];   // parent offset of logical (0, 0, 0)
    // Remove(padval): the rings hold padval for good, filled once; Wrap / Reflect: refreshed every step
    int rc = launch_grid_copy(a, 0, &pg[0], inner, n, s);
    const bool fixed_ring = bc->boundary == STC_REMOVE;
    if (!rc && fixed_ring) rc = launch_halo_fill(&pg[0], R, &hb, s);
    if (!rc && fixed_ring) rc = launch_halo_fill(&pg[1], R, &hb, s);
    // Wrap / Reflect: the ring is refreshed (K2) before every step.  (Writing each output's ring images
    // from the map kernel instead measured slower on 512^3: 384 us per step against 188 + 41 us.)
    int cur = 0;
    for (int64_t k = 0; k < nsteps && !rc; ++k) {
        if (!fixed_ring && (rc = launch_halo_fill(&pg[cur], R, &hb, s))) break;
        if ((rc = launch_map(&pg[cur], &pg[1 - cur], 1, st, op, &hb, s, ctx))) break;
        cur = 1 - cur;
    }
    const bool res_in_b = (nsteps & 1) != 0;
    if (!rc) rc = launch_grid_copy(&pg[cur], inner, res_in_b ? b : a, 0, n, s);
    if (!rc) rc = launch_grid_copy(&pg[1 - cur], inner, res_in_b ? a : b, 0, n, s);
    workspace_release(mem, cached, s);
    if (rc) return rc;
    *src_is_b = res_in_b ? 1 : 0;
    *done = nsteps;
    return STC_OK;
}
// stc_map_steps with a padval of another type: every step reads the neighbours in the promoted type
// (the source parent converted), maps into a result of that type's result type, and converts it back
// into the dest parent, as the reference's setindex! does (InexactError where it is not exact).
static int map_steps_promoted(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op,
                              const stc_bc* bc, int ndt, int64_t nsteps, int32_t* out_src_is_b, void* stream,
                              uint32_t flags) {
    if (check_grid(b) || !st || !op) return STC_ERR_INVALID;
    for (int d = 0; d < a->ndims; ++d)
        if (a->size[d] != b->size[d] || a->dtype != b->dtype) return STC_ERR_SIZE_MISMATCH;
    const int rdt = result_dtype(op->code, ndt, st->weight_dtype);
    if (rdt < 0) return rdt;
    stc_grid fake = *a;   // the step's result: a parent of the result type
    fake.dtype = rdt;
    int rc = validate_map(a, &fake, 1, st, op, bc);
    if (rc) return rc;
    if (nsteps > 0 && grids_overlap(a, b)) return STC_ERR_INVALID;
    DeviceCtx* ctx = nullptr;
    if ((rc = device_ctx(&ctx))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int src_is_b = 0;
    if (nsteps > 0) {
        stc_grid tin, tout;
        if ((rc = dense_like(a, ndt, &tin, s))) return rc;
        if ((rc = dense_like(a, rdt, &tout, s))) { cudaFreeAsync(tin.data, s); return rc; }
        stc_bc b2 = *bc;
        b2.padval_type = 0;
        const bool halo = bc->padding != STC_CONDITIONAL;
        const int R = halo ? st->radius : 0;
        int64_t whole[3], n[3];
        sizes3(a, whole);
        for (int d = 0; d < 3; ++d) n[d] = d < a->ndims ? a->size[d] - 2 * R : 1;
        auto org = [&](const stc_grid* g) {
            int64_t o = 0;
            for (int d = 0; d < g->ndims; ++d) o += (int64_t)R * g->stride[d];
            return o;
        };
        const stc_grid* grids[2] = {a, b};
        for (int64_t k = 0; k < nsteps && !rc; ++k) {
            const stc_grid* sg = grids[src_is_b];
            const stc_grid* dg = grids[1 - src_is_b];
            rc = launch_grid_convert(sg, 0, &tin, 0, whole, status_slot(ctx, s).dev, s);
            if (!rc) rc = launch_halo_fill(&tin, st->radius, &b2, s);
            if (!rc) rc = launch_map(&tin, &tout, 1, st, op, &b2, s, ctx);
            if (!rc) rc = launch_grid_convert(&tout, org(&tout), dg, org(dg), n, status_slot(ctx, s).dev, s);
            src_is_b = 1 - src_is_b;
        }
        cudaFreeAsync(tin.data, s);
        cudaFreeAsync(tout.data, s);
        if (rc) return rc;
    }
    if (out_src_is_b) *out_src_is_b = src_is_b;
    return (flags & STC_ASYNC) ? STC_OK : finish_sync(s, ctx);
}

}  // namespace stc

extern "C" {

int stc_map_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op, const stc_bc* bc,
                  int64_t nsteps, int32_t* out_src_is_b, void* stream, uint32_t flags) {
    if (nsteps < 0) return STC_ERR_INVALID;
    if (check_grid(a) || !bc) return STC_ERR_INVALID;
    const int ndt = neighbor_dtype(a->dtype, bc);
    if (ndt < 0) return ndt;
    if (ndt != a->dtype) return map_steps_promoted(a, b, st, op, bc, ndt, nsteps, out_src_is_b, stream, flags);
    int rc = validate_map(a, b, 1, st, op, bc);
    if (rc) return rc;
    for (int d = 0; d < a->ndims; ++d)
        if (a->size[d] != b->size[d] || a->dtype != b->dtype) return STC_ERR_SIZE_MISMATCH;
    if (nsteps > 0 && grids_overlap(a, b)) return STC_ERR_INVALID;
    DeviceCtx* ctx = nullptr;
    if ((rc = device_ctx(&ctx))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    int64_t done = 0;
    int src_is_b = 0;
    // Cellular automata on bit-packable grids run temporally blocked on a packed copy.
    rc = life_try_steps(a, b, st, op, bc, nsteps, &src_is_b, s, ctx, &done);
    if (rc) return rc;
    // 3D radius-1 float maps: k steps per pass over HBM (temporal blocking)
    if (done == 0) {
        rc = tb3d_try_steps(a, b, st, op, bc, nsteps, &src_is_b, s, ctx, flags, &done);
        if (rc) return rc;
    }
    // 2D radius-1 Float32 maps: blocked passes of 4 steps, the last few steps per step below
    if (done == 0) {
        rc = tb2d_try_steps(a, b, st, op, bc, nsteps, &src_is_b, s, ctx, &done);
        if (rc) return rc;
    }
    if (done == 0 && (flags & STC_KEEP_F32) && (a->dtype == STC_BF16 || a->dtype == STC_F16) && nsteps > 0)
        return STC_ERR_UNSUPPORTED;
    // other 3D grids whose boundary needs edge patching: steps on an internal Halo-padded pair
    if (done == 0) {
        rc = padded_steps(a, b, st, op, bc, nsteps, &src_is_b, s, ctx, &done);
        if (rc) return rc;
    }
    const stc_grid* grids[2] = {a, b};
    for (int64_t k = done; k < nsteps; ++k) {
        const stc_grid* sg = grids[src_is_b];
        const stc_grid* dg = grids[1 - src_is_b];
        if ((rc = launch_halo_fill(sg, st->radius, bc, s))) return rc;
        if ((rc = launch_map(sg, dg, 1, st, op, bc, s, ctx))) return rc;
        src_is_b = 1 - src_is_b;
    }
    if (out_src_is_b) *out_src_is_b = src_is_b;
    if (!(flags & STC_ASYNC)) rc = finish_sync(s, ctx);
    return rc;
}

// Host <-> device copies of a grid whose device side may be a strided view (the interior of a Halo
// parent): one pitched copy (cudaMemcpy2DAsync; one per plane when the planes are not stacked at one
// pitch), or one linear copy when the rows are contiguous; no staging kernel.
static int host_grid_copy(const stc_grid* g, void* host, bool upload, void* stream, uint32_t flags) {
    int rc = check_grid(g);
    if (rc) return rc;
    if (!host) return STC_ERR_INVALID;
    const size_t es = (size_t)dtype_size(g->dtype);
    const size_t w = (size_t)g->size[0] * es;
    const size_t h = g->ndims >= 2 ? (size_t)g->size[1] : 1, d = g->ndims >= 3 ? (size_t)g->size[2] : 1;
    if (!w || !h || !d) return STC_OK;
    if (!g->data) return STC_ERR_INVALID;
    const size_t dpitch = g->ndims >= 2 ? (size_t)g->stride[1] * es : w;
    if (g->ndims >= 2 && dpitch < w) return STC_ERR_INVALID;
    if (g->ndims == 3 && (size_t)g->stride[2] != (size_t)g->stride[1] * h) {
        // planes not stacked at one pitch: one 2D copy per plane
        for (size_t z = 0; z < d && !rc; ++z) {
            char* dp = (char*)g->data + z * (size_t)g->stride[2] * es;
            char* hp = (char*)host + z * w * h;
            cudaError_t e = upload ? cudaMemcpy2DAsync(dp, dpitch, hp, w, w, h, cudaMemcpyHostToDevice, (cudaStream_t)stream)
                                   : cudaMemcpy2DAsync(hp, w, dp, dpitch, w, h, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
            rc = cuda_fail(e);
        }
    } else if (dpitch == w) {
        // contiguous rows: one linear copy (less host work to issue than a pitched one)
        cudaError_t e = upload ? cudaMemcpyAsync(g->data, host, w * h * d, cudaMemcpyHostToDevice, (cudaStream_t)stream)
                               : cudaMemcpyAsync(host, g->data, w * h * d, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
        rc = cuda_fail(e);
    } else {
        cudaError_t e = upload
            ? cudaMemcpy2DAsync(g->data, dpitch, host, w, w, h * d, cudaMemcpyHostToDevice, (cudaStream_t)stream)
            : cudaMemcpy2DAsync(host, w, g->data, dpitch, w, h * d, cudaMemcpyDeviceToHost, (cudaStream_t)stream);
        rc = cuda_fail(e);
    }
    if (rc) return rc;
    if (!(flags & STC_ASYNC)) rc = cuda_fail(cudaStreamSynchronize((cudaStream_t)stream));
    return rc;
}

int stc_grid_upload(const stc_grid* dst, const void* host, void* stream, uint32_t flags) {
    return host_grid_copy(dst, (void*)host, true, stream, flags);
}

int stc_grid_download(void* host, const stc_grid* src, void* stream, uint32_t flags) {
    return host_grid_copy(src, host, false, stream, flags);
}

int stc_update_boundary(const stc_grid* parent, int32_t radius, const stc_bc* bc, void* stream, uint32_t flags) {
    int rc = check_grid(parent);
    if (rc) return rc;
    if (!bc || radius < 0) return STC_ERR_INVALID;
    for (int d = 0; d < parent->ndims; ++d)
        if (!(radius < parent->size[d]) || parent->size[d] - 2 * radius < 0) return STC_ERR_RADIUS;
    DeviceCtx* ctx = nullptr;
    if ((rc = device_ctx(&ctx))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if ((rc = launch_halo_fill(parent, radius, bc, s))) return rc;
    if (!(flags & STC_ASYNC)) rc = finish_sync(s, ctx);
    return rc;
}

}  // extern "C"
