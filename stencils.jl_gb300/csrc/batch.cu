// batch.cu — K5: many independent SwitchingStencilArray loops in one persistent, graph-captured launch.
//
// No counterpart in the reference (each job there is its own `A = mapstencil!(f, A)` loop,
// src/gatherstencil.jl:77-83).  A job is (two parents, stencil, reduction, boundary, steps); the batch
// runs every job to completion in one launch:
//   * A grid that fits in shared memory twice runs resident: one CTA loads it with a ring of R cells,
//     performs every step in shared memory (refreshing the ring from the interior for Wrap, padval for
//     Remove), and writes the result once.
//   * Larger grids are split into tiles; a work item advances one tile by k steps (k per job) from a
//     tile plus a k*R halo in shared memory, the halo's validity shrinking by R per step.  Item
//     (job, round r) needs every tile of (job, round r-1): a per-(job, round) counter in global memory
//     polled with a bounded wait.  Items are claimed in one queue from an atomic ticket, round-major,
//     so the oldest unfinished item's inputs are always complete and the queue cannot deadlock.
//     Round r reads parent r%2 and writes parent (r+1)%2; reads go through L2 (ld.global.cg) because
//     other SMs wrote that parent.
//   * Each cell's fold is the single-map kernel's (the same op structs), so every job's result is
//     bit-identical to running it alone through stc_map_steps.
// stc_batch_plan picks (tile, k) per job with an autotuner that times candidates on scratch grids of
// the job's size class and caches the winner; the launch (counter reset + kernel) is captured into a
// CUDA graph that stc_batch_run replays.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <type_traits>
#include <vector>

#include "batch.h"
#include "dispatch.h"
#include "map_kernel.cuh"
#include "map_launch.cuh"
#include "profile.h"

namespace stc {






template <class T> __device__ __forceinline__ T pad_of(const BatchJob& j);
template <> __device__ __forceinline__ float pad_of<float>(const BatchJob& j) { return j.padf; }
template <> __device__ __forceinline__ __nv_bfloat16 pad_of<__nv_bfloat16>(const BatchJob& j) {
    return __float2bfloat16_rn(j.padf);
}
template <> __device__ __forceinline__ uint8_t pad_of<uint8_t>(const BatchJob& j) { return (uint8_t)j.padi; }

template <class T> __device__ __forceinline__ T ld_l2(const T* p) { return *(const volatile T*)p; }
template <> __device__ __forceinline__ float ld_l2<float>(const float* p) { return __ldcg(p); }

__device__ __forceinline__ int wrapi(int i, int n) {
    i %= n;
    return i < 0 ? i + n : i;
}

template <class T, class Op>
__device__ __forceinline__ T batch_cell(const T* c, int pw, const int8_t* so, const OpArgs& a) {
    typename Op::A acc;
    int k0 = 0;
    if constexpr (Op::kZeroInit) {
        acc = Op::first(c[0], 0);
    } else {
        acc = Op::first(c[so[1] * pw + so[0]], 0);
        k0 = 1;
    }
    for (int k = k0; k < a.L; ++k) acc = Op::step(acc, c[so[2 * k + 1] * pw + so[2 * k]], k, a);
    return Op::finish(acc, c[0], a);
}

// The same fold with a compile-time table (the generated shape), in table order.
template <class T, class Op, class Sh>
__device__ __forceinline__ T batch_cell_shape(const T* c, int pw, const OpArgs& a) {
    constexpr auto Tb = Sh::table;
    typename Op::A acc;
    if constexpr (Op::kZeroInit) acc = Op::first(c[0], 0);
#pragma unroll
    for (int k = 0; k < Sh::L; ++k) {
        const T v = c[Tb.o[k].y * pw + Tb.o[k].x];
        if (!Op::kZeroInit && k == 0) acc = Op::first(v, 0);
        else acc = Op::step(acc, v, k, a);
    }
    return Op::finish(acc, c[0], a);
}

template <class T, class Op, class Sh>
__device__ __forceinline__ T batch_fold(const T* c, int pw, const int8_t* so, const OpArgs& a) {
    if constexpr (Sh::kKind == STC_SHAPE_TABLE) return batch_cell<T, Op>(c, pw, so, a);
    else return batch_cell_shape<T, Op, Sh>(c, pw, a);
}

// Advance one tile of one job by it.steps steps (the whole grid when resident).
template <class T, class Op, class Sh>
__device__ void batch_item(const BatchJob& j, const BatchItem& it, unsigned char* smem, const int8_t* so,
                           const OpArgs& oa) {
    const int R = j.R;
    const int steps = it.steps;
    int x0, y0, tw, th, pad;
    if (j.resident) {
        x0 = 0; y0 = 0; tw = j.n0; th = j.n1; pad = R;
    } else {
        x0 = (it.tile % j.ntx) * j.tw; y0 = (it.tile / j.ntx) * j.th;
        tw = j.tw; th = j.th; pad = steps * R;
    }
    const int pw = tw + 2 * pad, ph = th + 2 * pad;
    T* b0 = (T*)smem;
    T* b1 = b0 + (size_t)pw * ph;
    const int src = j.resident ? 0 : (it.round & 1);
    const int dstb = j.resident ? (j.nsteps & 1) : ((it.round + 1) & 1);
    const T* sp = (const T*)j.buf[src] + j.org[src];
    const T pv = pad_of<T>(j);
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        for (int by = warp; by < ph; by += nwarps) {
            const int gy = y0 - pad + by;
            const bool wr = j.boundary == STC_WRAP;
            const int gyw = wr ? wrapi(gy, j.n1) : gy;
            const bool row_in = wr || (gy >= 0 && gy < j.n1);
            const T* srow = sp + (int64_t)gyw * j.sy[src];
            for (int bx = lane; bx < pw; bx += 32) {
                const int gx = x0 - pad + bx;
                T v;
                if (wr) v = ld_l2(srow + (gx >= 0 && gx < j.n0 ? gx : wrapi(gx, j.n0)));
                else if (row_in && gx >= 0 && gx < j.n0) v = ld_l2(srow + gx);
                else v = pv;
                b0[by * pw + bx] = v;
            }
        }
    }
    __syncthreads();
    for (int g = 0; g < steps; ++g) {
        const T* in = (g & 1) ? b1 : b0;
        T* out = (g & 1) ? b0 : b1;
        const int lx = j.resident ? R : R * (g + 1), ly = lx;
        const int hx = j.resident ? R + tw : pw - R * (g + 1), hy = j.resident ? R + th : ph - R * (g + 1);
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        for (int by = ly + warp; by < hy; by += nwarps) {
            const int gy = y0 - pad + by;
            const bool row_out = j.boundary != STC_WRAP && (gy < 0 || gy >= j.n1);
            for (int bx = lx + lane; bx < hx; bx += 32) {
                const int gx = x0 - pad + bx;
                T v;
                if (row_out || (j.boundary != STC_WRAP && (gx < 0 || gx >= j.n0))) v = pv;
                else v = batch_fold<T, Op, Sh>(in + by * pw + bx, pw, so, oa);
                out[by * pw + bx] = v;
            }
        }
        __syncthreads();
        if (j.resident && g + 1 < steps) {
            // refresh the ring of R cells around the resident grid from its new interior
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
            for (int by = warp; by < ph; by += nwarps) {
                const bool ring_row = by < R || by >= R + th;
                const int sy = wrapi(by - R, th) + R;
                for (int bx = lane; bx < pw; bx += 32) {
                    if (!ring_row && bx >= R && bx < R + tw) continue;
                    out[by * pw + bx] = j.boundary == STC_WRAP ? out[sy * pw + wrapi(bx - R, tw) + R] : pv;
                }
            }
            __syncthreads();
        }
    }
    const T* fin = (steps & 1) ? b1 : b0;
    T* dp = (T*)j.buf[dstb] + j.org[dstb];
    {
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
        const int nvx = min(tw, j.n0 - x0), nvy = min(th, j.n1 - y0);
        for (int ty = warp; ty < nvy; ty += nwarps) {
            T* drow = dp + (int64_t)(y0 + ty) * j.sy[dstb] + x0;
            const T* frow = fin + (ty + pad) * pw + pad;
            for (int tx = lane; tx < nvx; tx += 32) drow[tx] = frow[tx];
        }
    }
}

// ---------------------------------------------------------------------------- vector-column tiles
// Fields compute_shape_vec reads, for one tile of one job (weights held in registers: NW = L for
// kernelproduct shapes).
template <int NW> struct BatchTileP {
    int32_t bw, bh, ry, rz, padl, tw;
    int64_t n[3];
    void* dst;
    int64_t dst_org;
    int64_t dstr[3];
    int32_t L;
    uint32_t birth, survive;
    double alpha;
    float rcp_f;
    int32_t fastdiv_f;
    float Lf;
    double Ld;
    float alpha_f;
    float wf[NW];
    const double* w;
    uint32_t box_bytes;   // the staged box (bounds tests of the debug build)
    int32_t* status;
};

// Geometry of the vector-column tiles of the batched kernel (shared with the host planner).
template <class T> struct BatchVecGeom {
    static constexpr int XV = 4, VS = 8;
    static constexpr int TW = 32 * XV, TH = (kBatchThreads / 32) * VS;
};
template <class T, int R> struct BatchVecBox {
    using G = BatchVecGeom<T>;
    static constexpr int PA = (R + G::XV - 1) / G::XV * G::XV;
    static constexpr int V = 16 / (int)sizeof(T);
    static constexpr int BW = (2 * PA + G::TW + V - 1) / V * V;
    static constexpr int BH = G::TH + 2 * R;
};

// One step of one tile: the tile's box (tile + R, Conditional rules of the job's boundary) is read
// through L2 into shared memory, then reduced by the single-map kernel's vector-column code straight
// into the destination parent, so each cell's fold is the one stc_map_steps performs.
template <class T, class Op, class Sh>
__device__ void batch_tile_vec(const BatchJob& j, const BatchItem& it, unsigned char* smem, const float* sw,
                               const OpArgs& oa, int32_t* status) {
    using G = BatchVecGeom<T>;
    constexpr int R = Sh::kR;
    using B = BatchVecBox<T, R>;
    constexpr int BW = B::BW, BH = B::BH, PA = B::PA;
    const int x0 = (it.tile % j.ntx) * G::TW, y0 = (it.tile / j.ntx) * G::TH;
    const int src = it.round & 1, dstb = (it.round + 1) & 1;
    const T* sp = (const T*)j.buf[src] + j.org[src];
    const T pv = pad_of<T>(j);
    T* box = (T*)smem;
    const bool wr = j.boundary == STC_WRAP;
    constexpr int TOTAL = BW * BH;
    // 8 loads in flight per thread between stores (24 measured slower: 26.4 against 22.8 ms per batch)
    constexpr int UNR = 8;
    for (int i0 = 0; i0 < TOTAL; i0 += kBatchThreads * UNR) {
        T v[UNR];
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int i = i0 + u * kBatchThreads + threadIdx.x;
            v[u] = pv;
            if (i < TOTAL) {
                const int by = i / BW, bx = i - by * BW;
                int gy = y0 - R + by, gx = x0 - PA + bx;
                bool in = gy >= 0 && gy < j.n1 && gx >= 0 && gx < j.n0;
                if (!in && wr) {
                    gy = wrapi(gy, j.n1);
                    gx = wrapi(gx, j.n0);
                    in = true;
                }
                if (in) v[u] = ld_l2(sp + (int64_t)gy * j.sy[src] + gx);
            }
        }
#pragma unroll
        for (int u = 0; u < UNR; ++u) {
            const int i = i0 + u * kBatchThreads + threadIdx.x;
            if (i < TOTAL) box[i] = v[u];
        }
    }
    __syncthreads();
    constexpr int NW = std::is_same_v<Op, OpKdotF<T, T>> ? Sh::L : 1;
    BatchTileP<NW> p;
    p.bw = BW; p.bh = BH; p.ry = R; p.rz = 0; p.padl = PA; p.tw = G::TW;
    p.n[0] = j.n0; p.n[1] = j.n1; p.n[2] = 1;
    p.dst = j.buf[dstb];
    p.dst_org = j.org[dstb];
    p.dstr[0] = 1; p.dstr[1] = j.sy[dstb]; p.dstr[2] = 0;
    p.L = oa.L; p.birth = oa.birth; p.survive = oa.survive; p.alpha = oa.alpha; p.rcp_f = oa.rcp_f;
    p.fastdiv_f = oa.fastdiv_f; p.Lf = oa.Lf; p.Ld = oa.Ld; p.alpha_f = oa.alpha_f; p.w = nullptr;
    p.box_bytes = (uint32_t)(BW * BH * sizeof(T));
    p.status = status;
#pragma unroll
    for (int k = 0; k < NW; ++k) p.wf[k] = NW > 1 ? sw[k] : 0.f;
    compute_shape_vec<T, T, Op, Sh, G::XV, G::VS>(p, TileOrigin{x0, y0, 0}, box);
}

// reduction types the batched kernel runs
using OpF_Mean = OpMean<float, float, float>;
using OpF_Sum = OpSumF<float, float, float>;
using OpF_Kdot = OpKdotF<float, float>;
using OpF_Min = OpMinMaxF<float, float, float, false>;
using OpF_Max = OpMinMaxF<float, float, float, true>;
using OpF_Diffuse = OpDiffuse<float, float, float>;
using OpB_Mean = OpMean<__nv_bfloat16, __nv_bfloat16, float>;
using OpB_Sum = OpSumF<__nv_bfloat16, __nv_bfloat16, float>;
using OpB_Kdot = OpKdotF<__nv_bfloat16, __nv_bfloat16>;
using OpB_Diffuse = OpDiffuse<__nv_bfloat16, __nv_bfloat16, float>;
using OpU_Life = OpLife<uint8_t, uint8_t>;
using OpU_Sum = OpSumI<uint8_t, uint8_t, STC_U8>;

__global__ void __launch_bounds__(kBatchThreads) batch_kernel(const BatchDev d) {
    extern __shared__ __align__(16) unsigned char bsm[];
    __shared__ int s_item;
    __shared__ int8_t so[2 * kBatchMaxL];
    __shared__ float sw[kBatchMaxL];
    while (true) {
        __syncthreads();
        if (threadIdx.x == 0) s_item = atomicAdd(d.ticket, 1);
        __syncthreads();
        const int ii = s_item;
        if (ii >= d.nitems || *((volatile int*)d.abort_flag)) return;
        const BatchItem it = d.items[ii];
        const BatchJob j = d.jobs[it.job];
        if (threadIdx.x == 0 && it.round > 0) {
            volatile int* ctr = d.counters + j.counter_base + it.round - 1;
            const long long t0 = clock64();
            while (*ctr < j.tiles) {
                if (clock64() - t0 > 4000000000ll) {   // ~2 s: give up, flag, and stop the queue
                    atomicOr(d.status, DEV_ERR_TIMEOUT);
                    atomicExch(d.abort_flag, 1);
                    break;
                }
                __nanosleep(100);
            }
            __threadfence();
        }
        for (int i = threadIdx.x; i < j.L; i += blockDim.x) {
            so[2 * i] = d.offs[2 * (j.off_base + i)];
            so[2 * i + 1] = d.offs[2 * (j.off_base + i) + 1];
            sw[i] = d.wts[j.off_base + i];
        }
        __syncthreads();
        if (*((volatile int*)d.abort_flag)) return;
        OpArgs oa;
        oa.L = j.L;
        oa.birth = j.birth;
        oa.survive = j.survive;
        oa.alpha = j.alpha;
        oa.rcp_f = j.rcp_f;
        oa.Lf = (float)j.L;
        oa.Ld = (double)j.L;
        oa.alpha_f = (float)j.alpha;
        oa.fastdiv_f = j.fastdiv_f;
        oa.wf = sw;
        oa.w = nullptr;
        const int key = j.dtype * 16 + j.opv;
#define STC_B(DT, OPV, T, OP)                                                                   \
    case DT * 16 + OPV:                                                                         \
        batch_item<T, OP, TableShape>(j, it, bsm, so, oa);                                      \
        break;
#define STC_BS(DT, OPV, T, OP, KIND, RR)                                                        \
    if (key == DT * 16 + OPV && j.shape == KIND && j.R == RR) {                                 \
        batch_item<T, OP, Shape<KIND, RR, 2>>(j, it, bsm, so, oa);                              \
        goto item_done;                                                                         \
    }
#define STC_BV(DT, OPV, T, OP, KIND, RR)                                                        \
    if (key == DT * 16 + OPV && j.shape == KIND && j.R == RR && j.vec) {                        \
        batch_tile_vec<T, OP, Shape<KIND, RR, 2>>(j, it, bsm, sw, oa, d.status);                          \
        goto item_done;                                                                         \
    }
        // vector-column tiles (one step per round) for the shapes batched workloads use
        STC_BV(STC_F32, OPV_MEAN, float, OpF_Mean, STC_SHAPE_WINDOW, 1)
        STC_BV(STC_F32, OPV_MEAN, float, OpF_Mean, STC_SHAPE_CIRCLE, 3)
        STC_BV(STC_F32, OPV_SUM, float, OpF_Sum, STC_SHAPE_CROSS, 2)
        STC_BV(STC_F32, OPV_KDOT_F, float, OpF_Kdot, STC_SHAPE_WINDOW, 2)
        STC_BV(STC_BF16, OPV_MEAN, __nv_bfloat16, OpB_Mean, STC_SHAPE_WINDOW, 1)
        STC_BV(STC_BF16, OPV_MEAN, __nv_bfloat16, OpB_Mean, STC_SHAPE_CIRCLE, 3)
        STC_BV(STC_BF16, OPV_KDOT_F, __nv_bfloat16, OpB_Kdot, STC_SHAPE_WINDOW, 2)
        STC_BV(STC_BF16, OPV_MEAN, __nv_bfloat16, OpB_Mean, STC_SHAPE_CROSS, 2)
        STC_BV(STC_U8, OPV_LIFE, uint8_t, OpU_Life, STC_SHAPE_MOORE, 1)
        // compile-time tables for the shapes batched workloads use
        STC_BS(STC_F32, OPV_MEAN, float, OpF_Mean, STC_SHAPE_WINDOW, 1)
        STC_BS(STC_F32, OPV_MEAN, float, OpF_Mean, STC_SHAPE_CIRCLE, 3)
        STC_BS(STC_F32, OPV_SUM, float, OpF_Sum, STC_SHAPE_CROSS, 2)
        STC_BS(STC_F32, OPV_KDOT_F, float, OpF_Kdot, STC_SHAPE_WINDOW, 2)
        STC_BS(STC_BF16, OPV_MEAN, __nv_bfloat16, OpB_Mean, STC_SHAPE_WINDOW, 1)
        STC_BS(STC_BF16, OPV_MEAN, __nv_bfloat16, OpB_Mean, STC_SHAPE_CIRCLE, 3)
        STC_BS(STC_BF16, OPV_KDOT_F, __nv_bfloat16, OpB_Kdot, STC_SHAPE_WINDOW, 2)
        STC_BS(STC_U8, OPV_LIFE, uint8_t, OpU_Life, STC_SHAPE_MOORE, 1)
        switch (key) {
        STC_B(STC_F32, OPV_MEAN, float, OpF_Mean)
        STC_B(STC_F32, OPV_SUM, float, OpF_Sum)
        STC_B(STC_F32, OPV_KDOT_F, float, OpF_Kdot)
        STC_B(STC_F32, OPV_MIN, float, OpF_Min)
        STC_B(STC_F32, OPV_MAX, float, OpF_Max)
        STC_B(STC_F32, OPV_DIFFUSE, float, OpF_Diffuse)
        STC_B(STC_BF16, OPV_MEAN, __nv_bfloat16, OpB_Mean)
        STC_B(STC_BF16, OPV_SUM, __nv_bfloat16, OpB_Sum)
        STC_B(STC_BF16, OPV_KDOT_F, __nv_bfloat16, OpB_Kdot)
        STC_B(STC_BF16, OPV_DIFFUSE, __nv_bfloat16, OpB_Diffuse)
        STC_B(STC_U8, OPV_LIFE, uint8_t, OpU_Life)
        STC_B(STC_U8, OPV_SUM, uint8_t, OpU_Sum)
        default: break;
        }
#undef STC_B
#undef STC_BS
#undef STC_BV
    item_done:
        __syncthreads();
        if (!j.resident) {
            __threadfence();
            __syncthreads();
            if (threadIdx.x == 0) atomicAdd(d.counters + j.counter_base + it.round, 1);
        }
    }
}

bool batch_supported(int dtype, int opv) {
    switch (dtype * 16 + opv) {
    case STC_F32 * 16 + OPV_MEAN: case STC_F32 * 16 + OPV_SUM: case STC_F32 * 16 + OPV_KDOT_F:
    case STC_F32 * 16 + OPV_MIN: case STC_F32 * 16 + OPV_MAX: case STC_F32 * 16 + OPV_DIFFUSE:
    case STC_BF16 * 16 + OPV_MEAN: case STC_BF16 * 16 + OPV_SUM: case STC_BF16 * 16 + OPV_KDOT_F:
    case STC_BF16 * 16 + OPV_DIFFUSE: case STC_U8 * 16 + OPV_LIFE: case STC_U8 * 16 + OPV_SUM:
        return true;
    }
    return false;
}

}  // namespace stc

// ====================================================================== host side
namespace stc {


// a grid held twice below this runs resident (STC_BATCH_RESIDENT_KB overrides, a tuning knob); the
// launch's shared memory per CTA is the largest any job needs, so this also sets CTAs per SM: 32 KB
// keeps the launch at 3 CTAs per SM (register-limited) and measured 22.8 ms per 256-grid batch
// against 29.9 ms with 96 KB (2 CTAs per SM)
static size_t resident_smem_cap() {
    static const size_t cap = [] {
        const char* e = getenv("STC_BATCH_RESIDENT_KB");
        const long v = e ? atol(e) : 0;
        return (size_t)((v >= 8 && v <= 200) ? v : 32) * 1024;
    }();
    return cap;
}
constexpr size_t kTiledSmemCap = 200 * 1024;
// The launch's shared memory per CTA is the largest any job needs, so one job's geometry sets every
// job's occupancy: autotuner candidates stay within the vector tiles' boxes (38 KB), which keeps the
// launch at 3 CTAs per SM.  (Uncapped, the tuner picked deep k-step tiles that were fastest alone
// and made the 256-grid batch 33.6 ms instead of 22.8.)
constexpr size_t kTunedSmemCap = 40 * 1024;

static size_t tiled_smem(const BatchSpec& s, const Geometry& g) {
    const size_t es = dtype_size(s.a.dtype);
    return 2 * (size_t)(g.tw + 2 * g.k * s.R) * (g.th + 2 * g.k * s.R) * es;
}

// Vector-column tile geometry for the (dtype, reduction, shape, R) the kernel has a vector path for
// (the STC_BV list of batch_kernel); false otherwise.
static bool vec_geometry(const BatchSpec& s, int shape, int* tw, int* th, size_t* smem) {
    auto geo = [&](auto t, auto r) {
        using T = decltype(t);
        constexpr int R = decltype(r)::value;
        *tw = BatchVecGeom<T>::TW;
        *th = BatchVecGeom<T>::TH;
        *smem = (size_t)BatchVecBox<T, R>::BW * BatchVecBox<T, R>::BH * sizeof(T);
        return true;
    };
    using I1 = std::integral_constant<int, 1>;
    using I2 = std::integral_constant<int, 2>;
    using I3 = std::integral_constant<int, 3>;
    const int dt = s.a.dtype, opv = s.opv, R = s.R;
    if (dt == STC_F32) {
        if (opv == OPV_MEAN && shape == STC_SHAPE_WINDOW && R == 1) return geo(0.f, I1{});
        if (opv == OPV_MEAN && shape == STC_SHAPE_CIRCLE && R == 3) return geo(0.f, I3{});
        if (opv == OPV_SUM && shape == STC_SHAPE_CROSS && R == 2) return geo(0.f, I2{});
        if (opv == OPV_KDOT_F && shape == STC_SHAPE_WINDOW && R == 2) return geo(0.f, I2{});
    } else if (dt == STC_BF16) {
        const __nv_bfloat16 b{};
        if (opv == OPV_MEAN && shape == STC_SHAPE_WINDOW && R == 1) return geo(b, I1{});
        if (opv == OPV_MEAN && shape == STC_SHAPE_CIRCLE && R == 3) return geo(b, I3{});
        if (opv == OPV_KDOT_F && shape == STC_SHAPE_WINDOW && R == 2) return geo(b, I2{});
        if (opv == OPV_MEAN && shape == STC_SHAPE_CROSS && R == 2) return geo(b, I2{});
    } else if (dt == STC_U8) {
        if (opv == OPV_LIFE && shape == STC_SHAPE_MOORE && R == 1) return geo((uint8_t)0, I1{});
    }
    return false;
}

static size_t resident_smem(const BatchSpec& s) {
    const size_t es = dtype_size(s.a.dtype);
    return 2 * (size_t)(s.a.size[0] + 2 * s.R) * (s.a.size[1] + 2 * s.R) * es;
}

using TuneKey = std::tuple<int, int, int, int, int, int>;   // dtype, opv, L, R, boundary, size bucket
static std::mutex g_tune_mu;
static std::map<TuneKey, Geometry> g_tune_cache;

static TuneKey tune_key(const BatchSpec& s) {
    const double cells = (double)s.a.size[0] * (double)s.a.size[1];
    const int bucket = (int)std::floor(std::log2(std::max(cells, 1.0)));
    return TuneKey(s.a.dtype, s.opv, s.L, s.R, s.bc.boundary, bucket);
}

static Geometry default_geometry(const BatchSpec& s) {
    Geometry g{64, 32, s.R <= 1 ? 4 : (s.R == 2 ? 2 : 1)};
    g.k = (int)std::max<int64_t>(1, std::min<int64_t>(g.k, s.nsteps));
    while (g.k > 1 && tiled_smem(s, g) > kTiledSmemCap) --g.k;
    return g;
}

}  // namespace stc

namespace stc {

static void release_graph(stc_batch* b) {
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->exec = nullptr;
    b->graph = nullptr;
}

static inline size_t align_to(size_t x, size_t a) { return (x + a - 1) / a * a; }

// Build jobs, items and device tables, then capture (counter reset + kernel) as a graph.

static int autotune_spec(const BatchSpec& s, DeviceCtx* ctx, cudaStream_t stream, Geometry* out) {
    const TuneKey key = tune_key(s);
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        auto it = g_tune_cache.find(key);
        if (it != g_tune_cache.end()) { *out = it->second; return STC_OK; }
    }
    const int64_t n0 = s.a.size[0], n1 = s.a.size[1];
    const size_t es = dtype_size(s.a.dtype);
    const int64_t steps = std::min<int64_t>(s.nsteps, 16);
    std::vector<Geometry> cands;
    const int tws[] = {32, 64, 128};
    const int ths[] = {16, 32, 64};
    const int ks[] = {1, 2, 4, 8};
    for (int tw : tws)
        for (int th : ths)
            for (int k : ks) {
                Geometry g{tw, th, k};
                if (k > steps || tiled_smem(s, g) > kTunedSmemCap) continue;
                if (tw * th < 1024 || tw * th > 8192) continue;
                cands.push_back(g);
            }
    // the one-step vector-column tiles, where the shape has them, compete with the k-step tiles
    {
        int vtw = 0, vth = 0;
        size_t vsmem = 0;
        const int shape = table_matches_shape(s.shape, s.R, 2, s.offs.data(), s.L) ? s.shape : STC_SHAPE_TABLE;
        if (vec_geometry(s, shape, &vtw, &vth, &vsmem)) cands.push_back(Geometry{vtw, vth, 1, 1});
    }
    if (cands.empty()) { *out = default_geometry(s); return STC_OK; }
    // enough copies of the job to fill the GPU the way a loaded batch would
    const int64_t tiles = ((n0 + 63) / 64) * ((n1 + 31) / 32);
    const int copies = (int)std::max<int64_t>(1, std::min<int64_t>(8, (2 * ctx->num_sms + tiles - 1) / tiles));
    const size_t gbytes = (size_t)n0 * n1 * es;
    void* scratch = nullptr;
    cudaError_t e = cudaMalloc(&scratch, 2 * copies * gbytes);
    if (e != cudaSuccess) return cuda_fail(e);
    cudaMemsetAsync(scratch, 0, 2 * copies * gbytes, stream);
    cudaEvent_t t0, t1;
    cudaEventCreate(&t0);
    cudaEventCreate(&t1);
    Geometry best = cands[0];
    float best_ms = 1e30f;
    int rc = STC_OK;
    for (const Geometry& g : cands) {
        stc_batch trial;
        for (int c = 0; c < copies; ++c) {
            BatchSpec t = s;
            t.nsteps = steps;
            t.a.data = (char*)scratch + (size_t)(2 * c) * gbytes;
            t.b.data = (char*)scratch + (size_t)(2 * c + 1) * gbytes;
            t.a.stride[1] = t.b.stride[1] = n0;
            t.force_tw = g.vec ? 0 : g.tw;
            t.force_th = g.vec ? 0 : g.th;
            t.force_k = g.vec ? 0 : g.k;
            t.force_vec = g.vec;
            trial.specs.push_back(t);
        }
        if ((rc = batch_build(&trial, false, stream, ctx))) break;
        float ms = 1e30f;
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(t0, stream);
            cudaGraphLaunch(trial.exec, stream);
            cudaEventRecord(t1, stream);
            cudaEventSynchronize(t1);
            float m = 0.f;
            cudaEventElapsedTime(&m, t0, t1);
            if (rep > 0) ms = std::min(ms, m);
        }
        batch_free(&trial);
        if (ms < best_ms) { best_ms = ms; best = g; }
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(t1);
    cudaStreamSynchronize(stream);
    cudaFree(scratch);
    if (rc) return rc;
    {
        std::lock_guard<std::mutex> g(g_tune_mu);
        g_tune_cache[key] = best;
    }
    *out = best;
    return STC_OK;
}

int batch_build(stc_batch* b, bool autotune, cudaStream_t stream, DeviceCtx* ctx, bool capture) {
    const int nj = (int)b->specs.size();
    b->hjobs.assign(nj, BatchJob{});
    b->hitems.clear();
    b->hoffs.clear();
    b->hwts.clear();
    b->result_in_b.assign(nj, 0);
    b->ncounters = 0;
    b->planned_cell_steps = 0;
    size_t smem = 0;
    int max_rounds = 0;
    std::vector<BatchItem> resident_items;
    for (int i = 0; i < nj; ++i) {
        const BatchSpec& s = b->specs[i];
        BatchJob& j = b->hjobs[i];
        j.buf[0] = s.a.data;
        j.buf[1] = s.b.data;
        j.org[0] = j.org[1] = 0;
        j.sy[0] = s.a.stride[1];
        j.sy[1] = s.b.stride[1];
        j.n0 = (int32_t)s.a.size[0];
        j.n1 = (int32_t)s.a.size[1];
        j.dtype = s.a.dtype;
        j.opv = s.opv;
        j.boundary = s.bc.boundary;
        j.L = s.L;
        j.R = s.R;
        j.nsteps = (int32_t)s.nsteps;
        j.padf = (float)s.bc.padval;
        j.padi = (int32_t)s.bc.padval_int;
        j.alpha = s.op.alpha;
        j.birth = s.op.birth_mask;
        j.survive = s.op.survive_mask;
        j.rcp_f = (float)(1.0 / (double)s.L);
        j.fastdiv_f = (s.opv == OPV_MEAN && s.a.dtype != STC_F64 && is_float_dtype(s.a.dtype)) ? (int)fastdiv_f_exact(s.L) : 0;
        j.shape = table_matches_shape(s.shape, s.R, 2, s.offs.data(), s.L) ? s.shape : STC_SHAPE_TABLE;
        j.off_base = (int32_t)(b->hoffs.size() / 2);
        for (int k = 0; k < s.L; ++k) {
            b->hoffs.push_back((int8_t)s.offs[2 * k]);
            b->hoffs.push_back((int8_t)s.offs[2 * k + 1]);
            b->hwts.push_back(s.wts.empty() ? 0.f : (float)s.wts[k]);
        }
        b->planned_cell_steps += (double)j.n0 * j.n1 * s.nsteps;
        if (s.nsteps == 0) { j.rounds = 0; continue; }
        const bool forced = s.force_tw > 0 || s.force_vec;
        if (!forced && resident_smem(s) <= resident_smem_cap()) {
            j.resident = 1;
            j.tw = j.n0; j.th = j.n1; j.k = j.nsteps;
            j.ntx = j.nty = j.tiles = 1;
            j.rounds = 1;
            smem = std::max(smem, resident_smem(s));
            resident_items.push_back(BatchItem{i, 0, 0, j.nsteps});
            b->result_in_b[i] = (int)(s.nsteps & 1);
            continue;
        }
        int vtw = 0, vth = 0;
        size_t vsmem = 0;
        const bool has_vec = vec_geometry(s, j.shape, &vtw, &vth, &vsmem);
        // geometry: an autotuner trial's, else the autotuner's choice for the job's size class (cached
        // per class), else the vector tiles where the shape has them, else the default k-step tiles
        Geometry g{0, 0, 0};
        bool use_vec = false;
        if (s.force_vec) {
            use_vec = has_vec;
        } else if (forced) {
            g = Geometry{s.force_tw, s.force_th, s.force_k};
        } else if (autotune) {
            int rc = autotune_spec(s, ctx, stream, &g);
            if (rc) return rc;
            use_vec = has_vec && g.vec;
        } else {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune_cache.find(tune_key(s));
            if (it != g_tune_cache.end() && !(b->prefer_vec && has_vec)) {
                g = it->second;
                use_vec = has_vec && g.vec;
            } else {
                use_vec = has_vec;
            }
        }
        if (use_vec) {
            // one step per round on vector-column tiles
            j.resident = 0;
            j.vec = 1;
            j.tw = vtw; j.th = vth; j.k = 1;
            j.ntx = (j.n0 + vtw - 1) / vtw;
            j.nty = (j.n1 + vth - 1) / vth;
            j.tiles = j.ntx * j.nty;
            j.rounds = (int32_t)s.nsteps;
            j.counter_base = b->ncounters;
            b->ncounters += j.rounds;
            smem = std::max(smem, vsmem);
            max_rounds = std::max(max_rounds, j.rounds);
            b->result_in_b[i] = j.rounds & 1;
            continue;
        }
        if (g.tw <= 0 || g.vec) g = default_geometry(s);
        g.k = (int)std::max<int64_t>(1, std::min<int64_t>(g.k, s.nsteps));
        j.resident = 0;
        j.tw = g.tw; j.th = g.th; j.k = g.k;
        j.ntx = (j.n0 + g.tw - 1) / g.tw;
        j.nty = (j.n1 + g.th - 1) / g.th;
        j.tiles = j.ntx * j.nty;
        j.rounds = (int32_t)((s.nsteps + g.k - 1) / g.k);
        j.counter_base = b->ncounters;
        b->ncounters += j.rounds;
        smem = std::max(smem, tiled_smem(s, g));
        max_rounds = std::max(max_rounds, j.rounds);
        b->result_in_b[i] = j.rounds & 1;
    }
    // resident jobs first, longest first, so they overlap the tiled rounds
    std::sort(resident_items.begin(), resident_items.end(), [&](const BatchItem& x, const BatchItem& y) {
        const BatchJob &a = b->hjobs[x.job], &c = b->hjobs[y.job];
        return (double)a.n0 * a.n1 * a.nsteps * a.L > (double)c.n0 * c.n1 * c.nsteps * c.L;
    });
    b->hitems = resident_items;
    for (int r = 0; r < max_rounds; ++r)
        for (int i = 0; i < nj; ++i) {
            const BatchJob& j = b->hjobs[i];
            if (j.resident || r >= j.rounds) continue;
            const int steps = (int)std::min<int64_t>(j.k, (int64_t)j.nsteps - (int64_t)r * j.k);
            for (int t = 0; t < j.tiles; ++t) b->hitems.push_back(BatchItem{i, r, t, steps});
        }
    // device tables in one block: jobs | items | offs | wts | counters | ticket, abort
    const size_t s_jobs = align_to(sizeof(BatchJob) * std::max(1, nj), 256);
    const size_t s_items = align_to(sizeof(BatchItem) * std::max<size_t>(1, b->hitems.size()), 256);
    const size_t s_offs = align_to(std::max<size_t>(2, b->hoffs.size()), 256);
    const size_t s_wts = align_to(sizeof(float) * std::max<size_t>(1, b->hwts.size()), 256);
    const size_t s_ctr = align_to(sizeof(int) * (size_t)(b->ncounters + 2), 256);
    const size_t total = s_jobs + s_items + s_offs + s_wts + s_ctr;
    cudaError_t e;
    if (total > b->dmem_bytes) {
        if (b->dmem) cudaFree(b->dmem);
        b->dmem = nullptr;
        if ((e = cudaMalloc(&b->dmem, total)) != cudaSuccess) return cuda_fail(e);
        b->dmem_bytes = total;
    }
    char* base = (char*)b->dmem;
    BatchDev& d = b->dev;
    d.jobs = (const BatchJob*)base;
    d.items = (const BatchItem*)(base + s_jobs);
    d.offs = (const int8_t*)(base + s_jobs + s_items);
    d.wts = (const float*)(base + s_jobs + s_items + s_offs);
    d.counters = (int*)(base + s_jobs + s_items + s_offs + s_wts);
    d.ticket = d.counters + b->ncounters;
    d.abort_flag = d.ticket + 1;
    d.nitems = (int)b->hitems.size();
    b->slot = status_slot(ctx, b);   // each batch (and each serving tick) has its own slot
    d.status = b->slot.dev;
    if (nj) cudaMemcpyAsync((void*)d.jobs, b->hjobs.data(), sizeof(BatchJob) * nj, cudaMemcpyHostToDevice, stream);
    if (!b->hitems.empty())
        cudaMemcpyAsync((void*)d.items, b->hitems.data(), sizeof(BatchItem) * b->hitems.size(), cudaMemcpyHostToDevice, stream);
    if (!b->hoffs.empty()) cudaMemcpyAsync((void*)d.offs, b->hoffs.data(), b->hoffs.size(), cudaMemcpyHostToDevice, stream);
    if (!b->hwts.empty())
        cudaMemcpyAsync((void*)d.wts, b->hwts.data(), sizeof(float) * b->hwts.size(), cudaMemcpyHostToDevice, stream);
    if ((e = cudaStreamSynchronize(stream)) != cudaSuccess) return cuda_fail(e);
    // launch shape: persistent CTAs
    b->smem = std::max<size_t>(smem, 16);
    if ((e = cudaFuncSetAttribute(batch_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)b->smem)) != cudaSuccess)
        return cuda_fail(e);
    int per_sm = 0;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, batch_kernel, kBatchThreads, b->smem)) != cudaSuccess)
        return cuda_fail(e);
    if (per_sm < 1) return STC_ERR_UNSUPPORTED;
    b->grid = (int)std::max<int64_t>(1, std::min<int64_t>((int64_t)per_sm * ctx->num_sms, std::max(1, d.nitems)));
    b->planned = true;
    if (!capture) return STC_OK;
    // capture: reset counters and the ticket, run the queue
    release_graph(b);
    if (!b->cap_stream && (e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_fail(e);
    if ((e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal)) != cudaSuccess) return cuda_fail(e);
    cudaMemsetAsync(d.counters, 0, sizeof(int) * (size_t)(b->ncounters + 2), b->cap_stream);
    if (d.nitems > 0) batch_kernel<<<b->grid, kBatchThreads, b->smem, b->cap_stream>>>(d);
    if ((e = cudaStreamEndCapture(b->cap_stream, &b->graph)) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaGraphInstantiate(&b->exec, b->graph, 0)) != cudaSuccess) return cuda_fail(e);
    return STC_OK;
}

int batch_launch(stc_batch* b, cudaStream_t stream) {
    BatchDev& d = b->dev;
    cudaError_t e = cudaMemsetAsync(d.counters, 0, sizeof(int) * (size_t)(b->ncounters + 2), stream);
    if (e != cudaSuccess) return cuda_fail(e);
    if (d.nitems > 0) batch_kernel<<<b->grid, kBatchThreads, b->smem, stream>>>(d);
    return cuda_fail(cudaGetLastError());
}

void batch_free(stc_batch* b) {
    release_graph(b);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    if (b->dmem) cudaFree(b->dmem);
    b->cap_stream = nullptr;
    b->dmem = nullptr;
    b->dmem_bytes = 0;
}

}  // namespace stc

using namespace stc;

extern "C" {

int stc_batch_create(stc_batch** out) {
    if (!out) return STC_ERR_INVALID;
    *out = new stc_batch();
    return STC_OK;
}

int stc_batch_destroy(stc_batch* b) {
    if (!b) return STC_ERR_INVALID;
    batch_free(b);
    delete b;
    return STC_OK;
}

int stc_batch_add(stc_batch* b, const stc_grid* a, const stc_grid* bg, const stc_stencil* st, const stc_op* op,
                  const stc_bc* bc, int64_t nsteps) {
    if (!b || nsteps < 0) return STC_ERR_INVALID;
    int rc = validate_map(a, bg, 1, st, op, bc);
    if (rc) return rc;
    if (nsteps > 0 && grids_overlap(a, bg)) return STC_ERR_INVALID;
    if (a->ndims != 2 || st->ndims != 2 || bc->padding != STC_CONDITIONAL) return STC_ERR_UNSUPPORTED;
    if (!(bc->boundary == STC_REMOVE || bc->boundary == STC_WRAP)) return STC_ERR_UNSUPPORTED;
    if (st->len > kBatchMaxL || st->radius > kBatchMaxR) return STC_ERR_UNSUPPORTED;
    for (int d = 0; d < 2; ++d)
        if (a->size[d] != bg->size[d] || a->dtype != bg->dtype) return STC_ERR_SIZE_MISMATCH;
    if (a->size[0] < 1 || a->size[1] < 1) return STC_ERR_INVALID;
    BatchSpec s;
    s.a = *a;
    s.b = *bg;
    s.L = st->len;
    s.R = st->radius;
    s.wdt = st->weight_dtype;
    s.shape = st->shape;
    s.offs.assign(st->offsets, st->offsets + 2 * st->len);
    if (st->weights) s.wts.assign(st->weights, st->weights + st->len);
    s.op = *op;
    s.bc = *bc;
    s.nsteps = nsteps;
    switch (op->code) {
    case STC_OP_MEAN: s.opv = OPV_MEAN; break;
    case STC_OP_SUM: s.opv = OPV_SUM; break;
    case STC_OP_KDOT: s.opv = (a->dtype != STC_F64 && is_float_dtype(a->dtype) && st->weight_dtype == STC_F32) ? OPV_KDOT_F : OPV_KDOT_D; break;
    case STC_OP_MIN: s.opv = OPV_MIN; break;
    case STC_OP_MAX: s.opv = OPV_MAX; break;
    case STC_OP_LIFE: s.opv = OPV_LIFE; break;
    case STC_OP_DIFFUSE: s.opv = OPV_DIFFUSE; break;
    default: return STC_ERR_UNSUPPORTED;
    }
    if (!batch_supported(a->dtype, s.opv)) return STC_ERR_UNSUPPORTED;
    b->specs.push_back(s);
    b->planned = false;
    return (int)b->specs.size() - 1;
}

namespace stc {
// Device time of one launch of the batch's plan (prefer_vec or the tuned geometries) run on zeroed
// scratch copies of every job's grids, so the caller's data is untouched; < 0 when it cannot be timed.
static float batch_trial_ms(const stc_batch* b, bool prefer_vec, cudaStream_t stream, DeviceCtx* ctx) {
    // every scratch grid starts on a 256-byte boundary (grids of different element sizes share the block)
    auto grid_bytes = [](const BatchSpec& sp) {
        return align_to((size_t)sp.a.size[0] * sp.a.size[1] * dtype_size(sp.a.dtype), 256);
    };
    size_t total = 0;
    for (const BatchSpec& sp : b->specs) total += 2 * grid_bytes(sp);
    void* scratch = nullptr;
    if (total == 0 || cudaMalloc(&scratch, total) != cudaSuccess) {
        cudaGetLastError();
        return -1.f;
    }
    cudaMemsetAsync(scratch, 0, total, stream);
    stc_batch trial;
    trial.prefer_vec = prefer_vec;
    size_t off = 0;
    for (const BatchSpec& sp : b->specs) {
        BatchSpec t = sp;
        const size_t gb = grid_bytes(sp);
        t.a.data = (char*)scratch + off;
        t.b.data = (char*)scratch + off + gb;
        t.a.stride[1] = t.b.stride[1] = sp.a.size[0];
        off += 2 * gb;
        trial.specs.push_back(t);
    }
    float best = -1.f;
    if (batch_build(&trial, false, stream, ctx) == STC_OK) {
        cudaEvent_t e0, e1;
        cudaEventCreate(&e0);
        cudaEventCreate(&e1);
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(e0, stream);
            cudaGraphLaunch(trial.exec, stream);
            cudaEventRecord(e1, stream);
            cudaEventSynchronize(e1);
            float ms = 0.f;
            cudaEventElapsedTime(&ms, e0, e1);
            if (rep > 0 && (best < 0.f || ms < best)) best = ms;
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
    }
    batch_free(&trial);
    cudaStreamSynchronize(stream);
    cudaFree(scratch);
    return best;
}
}  // namespace stc

int stc_batch_plan(stc_batch* b, int32_t autotune, void* stream) {
    if (!b) return STC_ERR_INVALID;
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    b->prefer_vec = false;
    if (!autotune) return batch_build(b, false, s, ctx);
    // 1. per size class, the fastest tile geometry (cached); 2. for the whole batch, the tuned plan
    // against vector tiles everywhere they apply, each timed once on scratch copies (one job's
    // geometry sets the shared memory, so the occupancy, of every job in the launch)
    if ((rc = batch_build(b, true, s, ctx, false))) return rc;
    const float tuned = batch_trial_ms(b, false, s, ctx);
    const float vec = batch_trial_ms(b, true, s, ctx);
    b->prefer_vec = vec >= 0.f && (tuned < 0.f || vec < tuned);
    return batch_build(b, false, s, ctx);
}

int stc_batch_run(stc_batch* b, void* stream, uint32_t flags) {
    if (!b) return STC_ERR_INVALID;
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if (!b->planned && (rc = batch_build(b, false, s, ctx))) return rc;
    void* prof = prof_begin(s);
    cudaError_t e = cudaGraphLaunch(b->exec, s);
    double bytes = 0;
    for (const BatchSpec& sp : b->specs) bytes += 2.0 * dtype_size(sp.a.dtype) * sp.a.size[0] * sp.a.size[1] * sp.nsteps;
    prof_end(prof, s, "batch_kernel", bytes, b->planned_cell_steps);
    if (e != cudaSuccess) return cuda_fail(e);
    if (!(flags & STC_ASYNC)) {
        if ((e = cudaStreamSynchronize(s)) != cudaSuccess) return cuda_fail(e);
        if (b->slot.host && (rc = take_status(b->slot))) return rc;
    }
    return STC_OK;
}

int stc_batch_result(const stc_batch* b, int32_t idx, int32_t* out_src_is_b) {
    if (!b || !out_src_is_b || idx < 0 || idx >= (int)b->specs.size()) return STC_ERR_INVALID;
    if (!b->planned) return STC_ERR_BUSY;
    *out_src_is_b = b->result_in_b[idx];
    return STC_OK;
}

int stc_batch_run_sequential(stc_batch* b, void* stream) {
    if (!b) return STC_ERR_INVALID;
    for (const BatchSpec& s : b->specs) {
        stc_stencil st{};
        st.ndims = 2;
        st.len = s.L;
        st.radius = s.R;
        st.shape = s.shape;
        st.offsets = s.offs.data();
        st.weights = s.wts.empty() ? nullptr : s.wts.data();
        st.weight_dtype = s.wdt;
        int32_t in_b = 0;
        int rc = stc_map_steps(&s.a, &s.b, &st, &s.op, &s.bc, s.nsteps, &in_b, stream, 0);
        if (rc) return rc;
    }
    return STC_OK;
}

}  // extern "C"
