// tblock3d.cu — K6: temporally blocked multi-step maps on 3D grids (plane-streaming wavefront).
//
// Replaces k iterations of  A = mapstencil!(f, A)  (src/gatherstencil.jl:77-83) for 3D radius-1
// stencils with float state (the 7-point diffusion of VonNeumann(1,3), 3D Moore/Cross(1) means/sums).
//
// A CTA owns an (x, y) tile of TX x TY outputs with a k-cell halo and a chunk of z.  It streams the
// input planes z0-k .. z1+k-1 through a TMA ring in shared memory (cp.async.bulk.tensor.3d, one plane
// per copy, no multicast); after plane i lands, time level t = 1..k computes its plane i-t from the
// three level t-1 planes below, above and at it (each level keeps a 4-plane ring, skewed so one
// barrier per plane suffices), the valid region
// shrinking by one cell per level in x and y.  Level k planes are the outputs.  So one pass over HBM
// advances the grid k steps.  Wrap: cells outside the grid are wrapped copies and evolve like the
// cells they copy.  Remove: cells outside the grid are reset to padval at every level.  Every cell
// update is the single-map fold (same op structs), so results are bit-identical to k separate maps.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>
#include <vector>

#include "dispatch.h"
#include "map_launch.cuh"
#include "profile.h"
#include "tblock.h"

namespace stc {

constexpr int kTbThreads = 256;
constexpr int kTbRing0 = 6;          // input planes in flight (prefetch distance kTbRing0 - 3)
constexpr int kTbRingL = 4;          // planes kept per intermediate time level (skewed schedule)

struct TBParams {
    CUtensorMap tmap;                // source parent (rank 3)
    const void* src;
    void* dst;
    int64_t sst[3], dstr[3];
    int64_t src_org, dst_org;
    int64_t n[3];
    int32_t hx[3];                   // parent coordinate of logical 0 (R for Halo parents)
    int32_t boundary;
    double padf;
    int32_t k;                       // time levels this launch
    int32_t TX, TY, ZC;              // tile and z chunk
    int32_t PX, PY, padl;            // plane box (x pitch, rows) and shared-memory x of the tile's first column
    int32_t ntx, nty, nzc;
    uint32_t plane_bytes;            // PX*PY*sizeof(T) rounded to 128
    int32_t fixup;                   // edge tiles need patching after TMA
    int32_t aligned;                 // dst rows allow 4-element vector stores (vector variant)
    int32_t* status;
    // op parameters (the fields the op structs read)
    int32_t L;
    uint32_t birth, survive;
    double alpha;
    float rcp_f;
    int32_t fastdiv_f;
    float Lf;
    double Ld;
    float alpha_f;
    float wf[64];
    double w[64];
};

template <class T> __device__ __forceinline__ T tb_pad(const TBParams& p);
template <> __device__ __forceinline__ float tb_pad<float>(const TBParams& p) { return (float)p.padf; }
template <> __device__ __forceinline__ __nv_bfloat16 tb_pad<__nv_bfloat16>(const TBParams& p) {
    return __float2bfloat16_rn((float)p.padf);
}
template <> __device__ __forceinline__ double tb_pad<double>(const TBParams& p) { return p.padf; }

// i mod n for the coordinates a plane box can hold (within one period of the grid almost always)
__device__ __forceinline__ int64_t tb_wrap(int64_t i, int64_t n) {
    if (i < 0) i += n;
    else if (i >= n) i -= n;
    if (i < 0 || i >= n) {
        i %= n;
        if (i < 0) i += n;
    }
    return i;
}

// value of logical cell (x, y, z) for the plane fix-up (Conditional rules: Wrap or Remove)
template <class T>
__device__ __forceinline__ T tb_load(const TBParams& p, int64_t x, int64_t y, int64_t z) {
    const T* s = (const T*)p.src;
    if (p.boundary == STC_WRAP) {
        x = tb_wrap(x, p.n[0]);
        y = tb_wrap(y, p.n[1]);
        z = tb_wrap(z, p.n[2]);
    } else if (x < 0 || x >= p.n[0] || y < 0 || y >= p.n[1] || z < 0 || z >= p.n[2]) {
        return tb_pad<T>(p);
    }
    return s[p.src_org + x + y * p.sst[1] + z * p.sst[2]];
}

// fold of one cell from the three planes below / at / above it (compile-time table, table order)
template <class T, class Op, class Sh>
__device__ __forceinline__ T tb_fold(const T* lo, const T* mid, const T* hi, int PX, const TBParams& p) {
    constexpr auto Tb = Sh::table;
    typename Op::A acc;
    if constexpr (Op::kZeroInit) acc = Op::first(mid[0], 0);
#pragma unroll
    for (int k = 0; k < Sh::L; ++k) {
        const T* pl = Tb.o[k].z < 0 ? lo : (Tb.o[k].z > 0 ? hi : mid);
        const T v = pl[Tb.o[k].y * PX + Tb.o[k].x];
        if (!Op::kZeroInit && k == 0) acc = Op::first(v, 0);
        else acc = Op::step(acc, v, k, p);
    }
    return Op::finish(acc, mid[0], p);
}

// ---- vector columns: one work item = 4 adjacent cells of a plane row ----
// Which rows of the three planes the generated table reads, and whether it reads their x - 1 / x + 1,
// as compile-time bit masks over the 3 x 3 (z, y) rows (scalars, so device code never reads the table
// object itself at run time).
template <class Sh> struct TbUse {
    static constexpr unsigned mask(int dx, bool any_x) {
        unsigned m = 0;
        for (int k = 0; k < Sh::L; ++k)
            if (any_x || Sh::table.o[k].x == dx) m |= 1u << ((Sh::table.o[k].z + 1) * 3 + (Sh::table.o[k].y + 1));
        return m;
    }
    static constexpr unsigned kRows = mask(0, true), kXm = mask(-1, false), kXp = mask(1, false);
};

template <class V, class T> __device__ __forceinline__ V tb_widen(T v) {
    if constexpr (std::is_same_v<V, T>) return v;
    else return __bfloat162float(v);
}

// The four cells at shared-memory offset `off` (a multiple of 4) of level t from the level t-1 planes
// (lo, mid, hi): each row the table reads is one aligned 4-wide load, plus its left / right neighbour
// when the table reads x - 1 / x + 1; every cell then folds its neighbours in table order (the same
// op structs, widened as in the single-map vector kernel), so results equal the one-cell fold.
template <class T, class Op, class Sh>
__device__ __forceinline__ void tb_cells4(const T* lo, const T* mid, const T* hi, int off, int PX, const TBParams& p,
                                          T* res) {
    using OpV = typename Widen<Op>::type;
    using V = std::conditional_t<Widen<Op>::kWide, float, T>;
    using U = TbUse<Sh>;
    constexpr auto Tb = Sh::table;
    V w[3][3][6];
#pragma unroll
    for (int zz = 0; zz < 3; ++zz)
#pragma unroll
        for (int yy = 0; yy < 3; ++yy) {
            const unsigned bit = 1u << (zz * 3 + yy);
            if (!(U::kRows & bit)) continue;
            const T* pl = (zz == 0 ? lo : (zz == 1 ? mid : hi)) + off + (yy - 1) * PX;
            ld_row_vec<T, V, 4>(pl, &w[zz][yy][1]);
            if (U::kXm & bit) w[zz][yy][0] = tb_widen<V>(pl[-1]);
            if (U::kXp & bit) w[zz][yy][5] = tb_widen<V>(pl[4]);
        }
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        typename OpV::A acc;
        if constexpr (OpV::kZeroInit) acc = OpV::first(V(0), 0);
#pragma unroll
        for (int k = 0; k < Sh::L; ++k) {
            const V v = w[Tb.o[k].z + 1][Tb.o[k].y + 1][c + Tb.o[k].x + 1];
            if (!OpV::kZeroInit && k == 0) acc = OpV::first(v, 0);
            else acc = OpV::step(acc, v, k, p);
        }
        if (!(U::kRows & (1u << 4))) w[1][1][c + 1] = tb_widen<V>(mid[off + c]);   // the centre, if the table skipped it
        res[c] = OpV::finish(acc, w[1][1][c + 1], p);
    }
}

template <class T> __device__ __forceinline__ void sts4(T* d, const T* v) {
    if constexpr (sizeof(T) == 4) {
        uint4 u;
        memcpy(&u, v, 16);
        *(uint4*)d = u;
    } else {
        uint2 u;
        memcpy(&u, v, 8);
        *(uint2*)d = u;
    }
}

template <class T, class Op, class Sh, bool VEC>
__global__ void __launch_bounds__(kTbThreads) tb3d_kernel(const __grid_constant__ TBParams p) {
    extern __shared__ __align__(128) unsigned char tsm[];
    const int k = p.k, PX = p.PX, PY = p.PY;
    const size_t pb = p.plane_bytes;
    // layout: level-0 ring (kTbRing0 planes), levels 1..k-1 (kTbRingL planes each), mbarriers
    auto plane0 = [&](int j) { return (T*)(tsm + (size_t)(j % kTbRing0) * pb); };
    auto planeL = [&](int t, int j) {
        return (T*)(tsm + (size_t)(kTbRing0 + kTbRingL * (t - 1) + (j % kTbRingL)) * pb);
    };
    uint64_t* bars = (uint64_t*)(tsm + (size_t)(kTbRing0 + kTbRingL * (k - 1)) * pb);

    int64_t t_id = blockIdx.x;
    const int tx = (int)(t_id % p.ntx);
    t_id /= p.ntx;
    const int ty = (int)(t_id % p.nty);
    const int tz = (int)(t_id / p.nty);
    const int64_t x0 = (int64_t)tx * p.TX, y0 = (int64_t)ty * p.TY, z0 = (int64_t)tz * p.ZC;
    const int64_t z1 = min(z0 + p.ZC, p.n[2]);
    const int NI = (int)(z1 - z0) + 2 * k;          // input planes z0-k .. z1+k-1
    const bool wrapb = p.boundary == STC_WRAP;
    const T pv = tb_pad<T>(p);
    // input plane j covers z = z0 - k + j; TMA when it lies in the grid or Wrap maps it there
    auto plane_z = [&](int j) { return z0 - k + j; };
    auto issue = [&](int j) {
        const int64_t z = plane_z(j);
        uint64_t* bar = &bars[j % kTbRing0];
        if (!wrapb && (z < 0 || z >= p.n[2])) {
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
            return;
        }
        const int64_t zz = wrapb ? tb_wrap(z, p.n[2]) : z;
        mbar_arrive_expect_tx(bar, (uint32_t)((size_t)PX * PY * sizeof(T)));
        tma_load_3d(plane0(j), &p.tmap, bar, (int)(x0 + p.hx[0] - p.padl), (int)(y0 + p.hx[1] - k),
                    (int)(zz + p.hx[2]));
    };
    if (threadIdx.x == 0) {
        prefetch_tensormap(&p.tmap);
        for (int s = 0; s < kTbRing0; ++s) mbar_init(&bars[s], 1);
        fence_barrier_init();
    }
    __syncthreads();
    const int ahead = kTbRing0 - 3;
    if (threadIdx.x == 0)
        for (int j = 0; j < min(ahead, NI); ++j) issue(j);
    // region of the box holding real tile columns/rows
    const bool edge_xy = x0 - k < 0 || y0 - k < 0 || x0 + p.TX + k > p.n[0] || y0 + p.TY + k > p.n[1];
    // Skewed wavefront: at iteration i, level t computes its plane j = i - 2t + 1.  Level 1 reads
    // level-0 planes i-2 .. i (plane i just landed); level t >= 2 reads level t-1 planes j-1 .. j+1,
    // all finished in earlier iterations.  So every level of an iteration is independent of the
    // others and one barrier per iteration suffices.  Iterations continue past the last input plane
    // until level k has produced every output plane.
    const int iters = NI + 2 * k - 1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    for (int i = 0; i < iters; ++i) {
        if (i < NI) {
            if (threadIdx.x == 0 && i + ahead < NI) {
                fence_proxy_async();
                issue(i + ahead);
            }
            const bool ok = mbar_wait_bounded(&bars[i % kTbRing0], (uint32_t)((i / kTbRing0) & 1));
            if (!__syncthreads_and(ok)) {
                if (threadIdx.x == 0) {
                    atomicOr(p.status, DEV_ERR_TIMEOUT);
                    for (int j = i; j < min(i + ahead, NI); ++j)
                        mbar_wait_bounded(&bars[j % kTbRing0], (uint32_t)((j / kTbRing0) & 1), 100000000ll);
                }
                return;
            }
            // level-0 plane i: patch cells outside the grid (Wrap copies / Remove padval)
            T* P0 = plane0(i);
            const int64_t z = plane_z(i);
            const bool zout = z < 0 || z >= p.n[2];
            if (!wrapb && zout) {
                for (int c = threadIdx.x; c < PX * PY; c += blockDim.x) P0[c] = pv;
                fence_proxy_async();   // generic writes before a later TMA refill of this slot
                __syncthreads();
            } else if (p.fixup && edge_xy) {
                // rows outside in y: every cell (a warp per row); rows inside: only the x cells beyond
                // either end, one per thread so that their loads are in flight together
                const int64_t gx0 = x0 - p.padl;
                const int xl = (int)max((int64_t)0, min((int64_t)PX, -gx0));             // bx < xl: gx < 0
                const int xr0 = (int)max((int64_t)xl, min((int64_t)PX, p.n[0] - gx0));   // bx >= xr0: gx >= n0
                const int nxo = xl + (PX - xr0);
                for (int it = threadIdx.x; it < PY * nxo; it += blockDim.x) {
                    const int by = it / nxo, c = it - by * nxo;
                    const int64_t gy = y0 - k + by;
                    if (gy < 0 || gy >= p.n[1]) continue;
                    const int bx = c < xl ? c : xr0 + (c - xl);
                    P0[by * PX + bx] = tb_load<T>(p, gx0 + bx, gy, z);
                }
                for (int by = warp; by < PY; by += nwarps) {
                    const int64_t gy = y0 - k + by;
                    if (gy >= 0 && gy < p.n[1]) continue;
                    for (int bx = lane; bx < PX; bx += 32) P0[by * PX + bx] = tb_load<T>(p, gx0 + bx, gy, z);
                }
                fence_proxy_async();
                __syncthreads();
            }
        }
        for (int t = 1; t <= k; ++t) {
            const int j = i - 2 * t + 1;               // plane index at level t
            if (j < t || j > NI - 1 - t) continue;     // uniform across the CTA
            const T* lo = (t == 1) ? plane0(j - 1) : planeL(t - 1, j - 1);
            const T* mid = (t == 1) ? plane0(j) : planeL(t - 1, j);
            const T* hi = (t == 1) ? plane0(j + 1) : planeL(t - 1, j + 1);
            const int64_t z = plane_z(j);
            const int xa = p.padl - k + t, xb = p.padl + p.TX + k - t;
            const int ya = t, yb = p.TY + 2 * k - t;
            if constexpr (VEC) {
                // work items: 4-cell groups from the multiple of 4 at or below xa (the extra cells left
                // of the valid region are computed and never read); padl and PX leave a spare column
                // group on each side, so the x - 1 / x + 1 reads stay inside the plane.
                const bool last = t == k;
                const int gx0 = last ? p.padl : (xa & ~3);
                const int ngx = last ? (p.TX >> 2) : ((xb - gx0 + 3) >> 2);
                const int row0 = last ? k : ya, nrows = last ? p.TY : yb - ya;
                const int nit = ngx * nrows;
                const float inv = 1.0f / (float)ngx;
                const bool zout = z < 0 || z >= p.n[2];
                T* out = last ? nullptr : planeL(t, j);
                T* dst = (T*)p.dst;
                const int nvx = (int)min((int64_t)p.TX, p.n[0] - x0), nvy = (int)min((int64_t)p.TY, p.n[1] - y0);
                for (int it = threadIdx.x; it < nit; it += blockDim.x) {
                    const int r = __float2int_rz(((float)it + 0.5f) * inv);   // it / ngx, exact (ngx <= 64)
                    const int g = it - r * ngx;
                    const int by = row0 + r, bx = gx0 + 4 * g;
                    const int off = by * PX + bx;
                    T res[4];
                    tb_cells4<T, Op, Sh>(lo, mid, hi, off, PX, p, res);
                    if (!last) {
                        if (!wrapb) {
                            // Remove: cells outside the grid hold padval at every level
                            const int64_t gy = y0 - k + by, gxa = x0 - p.padl + bx;
                            const bool row_out = zout || gy < 0 || gy >= p.n[1];
                            if (row_out || gxa < 0 || gxa + 3 >= p.n[0]) {
#pragma unroll
                                for (int c = 0; c < 4; ++c)
                                    if (row_out || gxa + c < 0 || gxa + c >= p.n[0]) res[c] = pv;
                            }
                        }
                        sts4<T>(out + off, res);
                    } else {
                        const int ly = r, lx = 4 * g;
                        if (ly < nvy && lx < nvx)
                            st_row_vec<T, 4>(dst + p.dst_org + z * p.dstr[2] + (y0 + ly) * p.dstr[1] + x0 + lx, res,
                                             p.aligned != 0, nvx - lx);
                    }
                }
                continue;
            }
            if (t < k) {
                T* out = planeL(t, j);
                const bool zout = z < 0 || z >= p.n[2];
                for (int by = ya + warp; by < yb; by += nwarps) {
                    const int64_t gy = y0 - k + by;
                    const bool row_out = !wrapb && (zout || gy < 0 || gy >= p.n[1]);
                    for (int bx = xa + lane; bx < xb; bx += 32) {
                        const int off = by * PX + bx;
                        const int64_t gx = x0 - p.padl + bx;
                        T v;
                        if (row_out || (!wrapb && (gx < 0 || gx >= p.n[0]))) v = pv;
                        else v = tb_fold<T, Op, Sh>(lo + off, mid + off, hi + off, PX, p);
                        out[off] = v;
                    }
                }
            } else {
                // level k: the outputs, tile interior only
                T* dst = (T*)p.dst;
                const int nvx = (int)min((int64_t)p.TX, p.n[0] - x0), nvy = (int)min((int64_t)p.TY, p.n[1] - y0);
                T* dplane = dst + p.dst_org + z * p.dstr[2] + x0;
                for (int ly = warp; ly < nvy; ly += nwarps) {
                    T* drow = dplane + (y0 + ly) * p.dstr[1];
                    for (int lx = lane; lx < nvx; lx += 32) {
                        const int off = (ly + k) * PX + lx + p.padl;
                        drow[lx] = tb_fold<T, Op, Sh>(lo + off, mid + off, hi + off, PX, p);
                    }
                }
            }
        }
        __syncthreads();
    }
}

// ------------------------------------------------------------------ host
typedef CUresult (*TbEncodeFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                               const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                               CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static TbEncodeFn tb_encoder() {
    static TbEncodeFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* q = nullptr;
        cudaDriverEntryPointQueryResult r;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &q, 12000, cudaEnableDefault, &r) ==
                cudaSuccess && r == cudaDriverEntryPointSuccess)
            fn = (TbEncodeFn)q;
    });
    return fn;
}

using TbLaunch = cudaError_t (*)(const TBParams&, int grid, size_t smem, cudaStream_t);

template <class T, class Op, class Sh, bool VEC>
static cudaError_t tb_launch_v(const TBParams& p, int grid, size_t smem, cudaStream_t s) {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [&] {
        attr = cudaFuncSetAttribute(tb3d_kernel<T, Op, Sh, VEC>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    });
    if (attr != cudaSuccess) return attr;
    tb3d_kernel<T, Op, Sh, VEC><<<grid, kTbThreads, smem, s>>>(p);
    return cudaGetLastError();
}

// the vector variant for Conditional grids (tile columns on 16-byte boundaries), else one cell per lane
template <class T, class Op, class Sh>
static cudaError_t tb_launch(const TBParams& p, int grid, size_t smem, cudaStream_t s) {
    return (p.hx[0] % 4 == 0 && p.padl % 4 == 0) ? tb_launch_v<T, Op, Sh, true>(p, grid, smem, s)
                                                  : tb_launch_v<T, Op, Sh, false>(p, grid, smem, s);
}

struct TbEntry { int dt, opv, shape; TbLaunch fn; };

static const TbEntry kTbTable[] = {
    {STC_F32, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, &tb_launch<float, OpDiffuse<float, float, float>, Shape<STC_SHAPE_VONNEUMANN, 1, 3>>},
    {STC_BF16, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN,
     &tb_launch<__nv_bfloat16, OpDiffuse<__nv_bfloat16, __nv_bfloat16, float>, Shape<STC_SHAPE_VONNEUMANN, 1, 3>>},
    {STC_F32, OPV_MEAN, STC_SHAPE_VONNEUMANN, &tb_launch<float, OpMean<float, float, float>, Shape<STC_SHAPE_VONNEUMANN, 1, 3>>},
    {STC_F32, OPV_MEAN, STC_SHAPE_MOORE, &tb_launch<float, OpMean<float, float, float>, Shape<STC_SHAPE_MOORE, 1, 3>>},
    {STC_F32, OPV_SUM, STC_SHAPE_CROSS, &tb_launch<float, OpSumF<float, float, float>, Shape<STC_SHAPE_CROSS, 1, 3>>},
};

static CUtensorMapDataType tb_dtype(int dt) {
    return dt == STC_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
}

int tb3d_try_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op, const stc_bc* bc,
                   int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx, int64_t* done) {
    *done = 0;
    if (nsteps < 3 || a->ndims != 3 || st->ndims != 3 || st->radius != 1) return STC_OK;
    // Opt-in (STC_TBLOCK=1): at its present instruction count per cell update the blocked kernel is
    // slower on GB300 than one K1 pass per step, which runs near the HBM roofline.
    const char* e = getenv("STC_TBLOCK");
    if (!(e && e[0] == '1')) return STC_OK;
    if (!(bc->boundary == STC_WRAP || bc->boundary == STC_REMOVE)) return STC_OK;
    int opv = op->code == STC_OP_DIFFUSE ? OPV_DIFFUSE : op->code == STC_OP_MEAN ? OPV_MEAN
              : op->code == STC_OP_SUM ? OPV_SUM : -1;
    TbLaunch fn = nullptr;
    for (const TbEntry& e : kTbTable)
        if (e.dt == a->dtype && e.opv == opv && table_matches_shape(e.shape, 1, 3, st->offsets, st->len)) fn = e.fn;
    if (!fn || !tb_encoder()) return STC_OK;
    const int es = dtype_size(a->dtype), V = 16 / es;
    for (const stc_grid* g : {a, b}) {
        if ((uintptr_t)g->data % 16) return STC_OK;
        for (int d = 1; d < 3; ++d)
            if ((g->stride[d] * es) % 16) return STC_OK;
    }
    const bool halo = bc->padding != STC_CONDITIONAL;
    TBParams p;
    memset(&p, 0, sizeof(p));
    for (int d = 0; d < 3; ++d) {
        p.n[d] = a->size[d] - (halo ? 2 : 0);
        p.hx[d] = halo ? 1 : 0;
        p.sst[d] = a->stride[d];
        p.dstr[d] = b->stride[d];
        if (p.n[d] < 1) return STC_OK;
    }
    p.boundary = bc->boundary;
    p.padf = bc->padval;
    p.status = ctx->status;
    p.L = st->len;
    p.alpha = op->alpha;
    p.rcp_f = (float)(1.0 / (double)st->len);
    p.fastdiv_f = (opv == OPV_MEAN && a->dtype != STC_F64) ? (int)fastdiv_f_exact(st->len) : 0;
    p.Lf = (float)st->len;
    p.Ld = (double)st->len;
    p.alpha_f = (float)op->alpha;
    p.TX = 64;
    p.TY = 16;
    const int smem_cap = 200 * 1024;
    // Halo parents are treated with the boundary applied on the fly (their rings are not refreshed
    // between the blocked steps); the patch after each plane copy covers every cell outside the grid.
    p.fixup = halo || !(bc->boundary == STC_REMOVE && bc->padval == 0.0 && !std::signbit(bc->padval));
    p.ntx = (int)((p.n[0] + p.TX - 1) / p.TX);
    p.nty = (int)((p.n[1] + p.TY - 1) / p.TY);
    const int64_t xy = (int64_t)p.ntx * p.nty;
    p.nzc = (int)std::max<int64_t>(1, std::min<int64_t>(p.n[2] / 32, (4 * ctx->num_sms + xy - 1) / xy));
    p.ZC = (int)((p.n[2] + p.nzc - 1) / p.nzc);
    p.nzc = (int)((p.n[2] + p.ZC - 1) / p.ZC);
    // launches: the first nsteps-1 steps, split so that state nsteps-1 ends in the parent the reference
    // leaves it in (a after an odd number of steps... i.e. m launches with m = nsteps-1 (mod 2))
    // deepest k <= 4 whose rings keep two CTAs per SM (<= 110 KB of shared memory)
    // Box geometry: the vector variant (Conditional grids, hx = 0) keeps the tile's first column at a
    // multiple of 4 and 16 bytes (padl = 8 >= k + 4) with room for its aligned 4-cell groups and their
    // x +- 1 reads on both sides; the one-cell variant needs only k columns of halo.
    const bool vec = p.hx[0] % 4 == 0;
    auto padl_for = [&](int kk) { return vec ? 8 : kk + (((p.hx[0] - kk) % V) + V) % V; };
    auto px_for = [&](int kk, int padl) { return (padl + p.TX + kk + (vec ? 7 : 0) + V - 1) / V * V; };
    int kmax = 4;
    {
        while (kmax > 1) {
            const int padl = padl_for(kmax);
            const int PX = px_for(kmax, padl);
            const size_t pbytes = ((size_t)PX * (p.TY + 2 * kmax) * es + 127) / 128 * 128;
            if ((size_t)(kTbRing0 + kTbRingL * (kmax - 1)) * pbytes <= 110 * 1024) break;
            --kmax;
        }
    }
    const int64_t blocked = nsteps - 1;
    int64_t m = (blocked + kmax - 1) / kmax;
    if ((m - blocked) % 2 != 0) ++m;
    if (m > blocked) m = blocked;
    std::vector<int> ks;
    for (int64_t i = 0; i < m; ++i) ks.push_back((int)(blocked / m + (i < blocked % m ? 1 : 0)));
    const stc_grid* par[2] = {a, b};
    int cur = *src_is_b;
    for (int kk : ks) {
        const stc_grid* sg = par[cur];
        const stc_grid* dg = par[1 - cur];
        p.k = kk;
        p.padl = padl_for(kk);
        p.PX = px_for(kk, p.padl);
        p.PY = p.TY + 2 * kk;
        p.plane_bytes = (uint32_t)(((size_t)p.PX * p.PY * es + 127) / 128 * 128);
        const size_t smem = (size_t)(kTbRing0 + kTbRingL * (kk - 1)) * p.plane_bytes + 8 * kTbRing0;
        if (smem > (size_t)smem_cap || p.PX > 256 || p.PY > 256) return *done ? STC_ERR_UNSUPPORTED : STC_OK;
        p.src = sg->data;
        p.dst = dg->data;
        p.src_org = halo ? 1 + sg->stride[1] + sg->stride[2] : 0;
        p.dst_org = halo ? 1 + dg->stride[1] + dg->stride[2] : 0;
        {
            const int VA = std::min(16, 4 * es);
            p.aligned = ((uintptr_t)dg->data + (uintptr_t)p.dst_org * es) % VA == 0 && (dg->stride[1] * es) % VA == 0 &&
                        (dg->stride[2] * es) % VA == 0;
        }
        for (int d = 0; d < 3; ++d) { p.sst[d] = sg->stride[d]; p.dstr[d] = dg->stride[d]; }
        cuuint64_t gdim[3] = {(cuuint64_t)sg->size[0], (cuuint64_t)sg->size[1], (cuuint64_t)sg->size[2]};
        cuuint64_t gstr[2] = {(cuuint64_t)(sg->stride[1] * es), (cuuint64_t)(sg->stride[2] * es)};
        cuuint32_t box[3] = {(cuuint32_t)p.PX, (cuuint32_t)p.PY, 1}, est[3] = {1, 1, 1};
        if (tb_encoder()(&p.tmap, tb_dtype(sg->dtype), 3, sg->data, gdim, gstr, box, est, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return *done ? STC_ERR_UNSUPPORTED : STC_OK;
        const int grid = p.ntx * p.nty * p.nzc;
        void* prof = prof_begin(stream);
        cudaError_t e = fn(p, grid, smem, stream);
        prof_end(prof, stream, "tblock3d", 2.0 * es * p.n[0] * p.n[1] * p.n[2] * kk, (double)p.n[0] * p.n[1] * p.n[2] * kk);
        if (e != cudaSuccess) return cuda_fail(e);
        cur = 1 - cur;
        *done += kk;
    }
    *src_is_b = cur;
    return STC_OK;
}

}  // namespace stc
