// tblock2d.cu — K7: temporally blocked multi-step maps on 2D Float32 grids.
//
// Replaces k iterations of  A = mapstencil!(f, A)  (src/gatherstencil.jl:77-83, switch src/array.jl:610-611)
// for 2D radius-1 stencils (Window(1), Moore(1), VonNeumann(1)) with the mean, sum and diffusion folds
// on Float32 state, under Wrap or Remove.
//
// Overlapped tiling: a CTA stages a box of 128 columns x BY rows of the source grid in shared memory
// (the tile of TX x TY outputs plus a halo of K cells on every side; cells beyond the grid edge
// are the wrapped cells under Wrap and padval under Remove), then computes K levels in a shared
// ping-pong pair: level g computes the box minus g cells on every side, so the last level is exactly
// the tile, which it writes straight to the destination parent.  One read and one write of HBM per
// cell and pass instead of per step; the recomputed halo costs about 17% of the updates at K = 8.
//
// Every thread owns one box column of one of the two row strips.  A strip streams down its column:
// each incoming row is read once from shared memory as its three (x-1, x, x+1) words and folded into
// the D = 3 outputs that use it, in the order of the stencil's offset table (rows ascending, then
// columns), so every output's fold is the single map's fold and the result is bit-identical to K
// separate maps.  Cells outside the grid under Remove are written as padval at every level, as
// getneighbor returns it at every step (src/array.jl:129-137); under Wrap the box's out-of-grid cells
// are copies of grid cells and evolve exactly like them.  The mean's correctly rounded division uses the
// FMA-corrected quotient; a tile whose staged values all lie where that quotient is exact at every level
// skips the per-output range test (T2Range).
#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <type_traits>

#include "dispatch.h"
#include "map_kernel.cuh"
#include "profile.h"
#include "tblock.h"

namespace stc {

constexpr int kT2Threads = 256;
constexpr int kT2BX = 128;                    // box columns: one per thread of a strip
constexpr int kT2Strips = kT2Threads / kT2BX;

struct TB2Params {
    const float* src;      // source parent, element of logical (0, 0)
    float* dst;            // destination parent, element of logical (0, 0)
    int64_t sstr, dstr;    // row strides (elements)
    int32_t n0, n1;        // logical size
    int32_t BY;            // box rows
    int32_t TX, TY;        // tile outputs (TX = 128 - 2K, TY = BY - 2K)
    int32_t ntx, ntiles;
    int32_t* status;       // debug build: bounds tests
    int32_t remove;        // Remove: cells outside the grid hold padval at every level
    int32_t vec_ok;        // interior boxes may be staged with 16-byte loads
    float padf;
    // the fields the op structs read
    int32_t L;
    uint32_t birth, survive;
    double alpha;
    float rcp_f;
    int32_t fastdiv_f;
    float Lf;
    double Ld;
    float alpha_f;
};

__device__ __forceinline__ int t2_wrap(int i, int n) {
    i %= n;
    return i < 0 ? i + n : i;
}

// Range of the staged values for the mean's division: true if every value this thread staged is +0 or
// lies in [2^-64, 2^124].  Then every sum formed over K <= 8 levels of means of at most 9 such values is 0
// or within [2^-90, 3e38], where the FMA-corrected quotient (div_by_len's fast branch) is exact, so the
// per-output range test can be dropped for the tile.
struct T2Range {
    uint32_t lo = 0xffffffffu, hi = 0u;   // min of (bits - 1) (a +0 wraps to the top), max of bits
    __device__ __forceinline__ void add(float v) {
        const uint32_t b = __float_as_uint(v);
        lo = min(lo, b - 1u);
        hi = max(hi, b);
    }
    __device__ __forceinline__ bool ok() const { return lo >= 0x1F7FFFFFu && hi <= 0x7D800000u; }
};

// Stage box rows [0, BY) x columns [0, 128) whose cell (0, 0) is grid cell (gx0, gy0).
__device__ __forceinline__ void t2_load_box(const TB2Params& p, float* box, int gx0, int gy0, bool inside, T2Range& rg) {
    const int BY = p.BY;
    if (inside && p.vec_ok) {
        // 32 float4 per row; gx0 is a multiple of 4 and so is the row stride
        for (int i = threadIdx.x; i < 32 * BY; i += blockDim.x) {
            const int r = i >> 5, c4 = i & 31;
            const float4 v = __ldg((const float4*)(p.src + (int64_t)(gy0 + r) * p.sstr + gx0) + c4);
            *((float4*)(box + r * kT2BX) + c4) = v;
            rg.add(v.x);
            rg.add(v.y);
            rg.add(v.z);
            rg.add(v.w);
        }
    } else if (inside) {
        for (int i = threadIdx.x; i < kT2BX * BY; i += blockDim.x) {
            const int r = i >> 7, c = i & 127;
            box[i] = __ldg(p.src + (int64_t)(gy0 + r) * p.sstr + gx0 + c);
            rg.add(box[i]);
        }
    } else {
        for (int i = threadIdx.x; i < kT2BX * BY; i += blockDim.x) {
            const int r = i >> 7, c = i & 127;
            int gx = gx0 + c, gy = gy0 + r;
            float v;
            if (p.remove) {
                v = (gx >= 0 && gx < p.n0 && gy >= 0 && gy < p.n1) ? __ldg(p.src + (int64_t)gy * p.sstr + gx) : p.padf;
            } else {
                gx = t2_wrap(gx, p.n0);
                gy = t2_wrap(gy, p.n1);
                v = __ldg(p.src + (int64_t)gy * p.sstr + gx);
            }
            box[i] = v;
            rg.add(v);
        }
    }
}

// One strip of one level: outputs (x, y) for y in [ra, rb) from the level below in `cur`.  LAST: the
// outputs are the tile's and go to the destination parent (column pointer gcol, row gy0 + y, rows
// below n1 only); else they go to `oth`, as padval where `patch` says the cell is outside the grid.
template <class Op, class Sh, bool LAST, bool FASTQ>
__device__ __forceinline__ void t2_strip(const TB2Params& p, const float* cur, float* oth, int x, int ra, int rb,
                                         bool patch, bool xin, int gy0, float* gcol) {
    constexpr int R = Sh::kR, D = 2 * R + 1, L = Sh::L;
    constexpr auto T = Sh::table;
    static_assert(T.o[0].y == -R, "tables start at the lowest row offset");
    using A = typename Op::A;
    A acc[D];
    float ctr[D];
#pragma unroll
    for (int q = 0; q < D; ++q) {
        acc[q] = A(0);
        ctr[q] = 0.f;
    }
    const float* col = cur + x - R;   // row r, column offset xx - R: col[r * 128 + xx]
    auto fold = [&](const float (&v)[D], const int q, const int slot) {
        // the row at offset q - R of the output held in `slot`
        if (Op::kZeroInit && q == 0) acc[slot] = Op::first(0.f, 0);
#pragma unroll
        for (int k = 0; k < L; ++k) {
            if (T.o[k].y != q - R) continue;
            const float val = v[T.o[k].x + R];
            if (!Op::kZeroInit && k == 0) acc[slot] = Op::first(val, 0);
            else acc[slot] = Op::step(acc[slot], val, k, p);
        }
        if (Op::kNeedsCentre && q == R) ctr[slot] = v[R];
    };
    auto finish = [&](const int slot, const int y) {
        float out;
        if constexpr (FASTQ) {
            // the mean's quotient without the range test (the tile's range was checked when staged)
            const float a = acc[slot];
            const float q = __fmul_rn(a, p.rcp_f);
            const float e = __fmaf_rn(-q, p.Lf, a);
            out = __fmaf_rn(e, p.rcp_f, q);
        } else if constexpr (std::is_same_v<Op, OpMean<float, float, A>>) {
            out = Op::template finish_c<L>(acc[slot], ctr[slot], p);
        } else {
            out = Op::finish(acc[slot], ctr[slot], p);
        }
        if constexpr (LAST) {
            if (gy0 + y < p.n1) gcol[(int64_t)(gy0 + y) * p.dstr] = out;
        } else {
            if (patch) {
                const int gy = gy0 + y;
                if (!xin || gy < 0 || gy >= p.n1) out = p.padf;
            }
            oth[y * kT2BX + x] = out;
        }
    };
    // prologue: rows ra-R .. ra+R-1 start the first outputs (output ra + i - q sits in slot (i - q) mod D)
#pragma unroll
    for (int i = 0; i < 2 * R; ++i) {
        float v[D];
#pragma unroll
        for (int xx = 0; xx < D; ++xx) v[xx] = col[(ra - R + i) * kT2BX + xx];
#pragma unroll
        for (int q = 0; q <= i; ++q) fold(v, q, (i - q) % D);
    }
    // steady state: row y + R completes output y (slot (y - ra) mod D) and feeds the next 2R outputs; whole
    // groups of D outputs first, then the last 0 .. D-1
    auto output = [&](const int j, const int y) {
        float v[D];
#pragma unroll
        for (int xx = 0; xx < D; ++xx) v[xx] = col[(y + R) * kT2BX + xx];
#pragma unroll
        for (int q = 0; q < D; ++q) fold(v, q, (j + 2 * R - q) % D);
        finish(j, y);
    };
    const int yfull = ra + (rb - ra) / D * D;
    int y0 = ra;
    for (; y0 < yfull; y0 += D) {
#pragma unroll
        for (int j = 0; j < D; ++j) output(j, y0 + j);
    }
#pragma unroll
    for (int j = 0; j < D - 1; ++j)
        if (y0 + j < rb) output(j, y0 + j);
}

template <class Op, class Sh, int K>
__global__ void __launch_bounds__(kT2Threads) tb2_kernel(const TB2Params p) {
    extern __shared__ __align__(16) float t2sm[];
    constexpr int R = Sh::kR;
    static_assert(R == 1, "the box halo is K cells");
    static_assert(K <= 8 && Sh::L <= 9, "the staged-range test assumes at most 8 levels of at most 9 taps");
    constexpr bool kMean = std::is_same_v<Op, OpMean<float, float, float>>;
    const int BY = p.BY;
    float* const buf0 = t2sm;
    float* const buf1 = t2sm + kT2BX * BY;
    const int x = threadIdx.x & (kT2BX - 1), s = threadIdx.x / kT2BX;
    for (int tile = blockIdx.x; tile < p.ntiles; tile += gridDim.x) {
        const int tx = tile % p.ntx, ty = tile / p.ntx;
        const int gx0 = tx * p.TX - K, gy0 = ty * p.TY - K;   // grid cell of box (0, 0)
        const bool inside = gx0 >= 0 && gy0 >= 0 && gx0 + kT2BX <= p.n0 && gy0 + BY <= p.n1;
        __syncthreads();   // the previous tile's last level has read buf0 / buf1
        T2Range rg;
        t2_load_box(p, buf0, gx0, gy0, inside, rg);
        const bool fastq = __syncthreads_and(rg.ok()) && kMean && p.fastdiv_f;
        const bool patch = p.remove && !inside;
        const int gx = gx0 + x;
        const bool xin = gx >= 0 && gx < p.n0;
        const float* cur = buf0;
        float* oth = buf1;
#pragma unroll 1
        for (int g = 1; g < K; ++g) {
            const int lo = g * R, nr = BY - 2 * g * R;
            const int ra = lo + nr * s / kT2Strips, rb = lo + nr * (s + 1) / kT2Strips;
            // the strip reads box rows ra-1 .. rb and columns x-1 .. x+1 (debug build: tested against the box)
            if (x >= g * R && x < kT2BX - g * R && STC_IN_BOUNDS(ra - 1, BY, p.status) && STC_IN_BOUNDS(rb, BY, p.status) &&
                STC_IN_BOUNDS(x - 1, kT2BX, p.status) && STC_IN_BOUNDS(x + 1, kT2BX, p.status)) {
                if (kMean && fastq) t2_strip<Op, Sh, false, kMean>(p, cur, oth, x, ra, rb, patch, xin, gy0, nullptr);
                else t2_strip<Op, Sh, false, false>(p, cur, oth, x, ra, rb, patch, xin, gy0, nullptr);
            }
            __syncthreads();
            const float* t = cur;
            cur = oth;
            oth = (float*)t;
        }
        {
            const int lo = K * R, nr = BY - 2 * K * R;
            const int ra = lo + nr * s / kT2Strips, rb = lo + nr * (s + 1) / kT2Strips;
            if (x >= K * R && x < kT2BX - K * R && gx < p.n0 && STC_IN_BOUNDS(ra - 1, BY, p.status) &&
                STC_IN_BOUNDS(rb, BY, p.status)) {
                if (kMean && fastq) t2_strip<Op, Sh, true, kMean>(p, cur, nullptr, x, ra, rb, false, true, gy0, p.dst + gx);
                else t2_strip<Op, Sh, true, false>(p, cur, nullptr, x, ra, rb, false, true, gy0, p.dst + gx);
            }
        }
    }
}

using Tb2Launch = cudaError_t (*)(const TB2Params&, int grid, size_t smem, cudaStream_t);

template <class Op, class Sh, int K>
static cudaError_t tb2_launch(const TB2Params& p, int grid, size_t smem, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(tb2_kernel<Op, Sh, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    tb2_kernel<Op, Sh, K><<<grid, kT2Threads, smem, s>>>(p);
    return cudaGetLastError();
}

template <class Op, class Sh, int K>
static cudaError_t tb2_occupancy(size_t smem, int* blocks) {
    cudaError_t e = cudaFuncSetAttribute(tb2_kernel<Op, Sh, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, tb2_kernel<Op, Sh, K>, kT2Threads, smem);
}

struct Tb2Entry {
    int opv, shape;
    Tb2Launch fn4, fn8;
    cudaError_t (*occ4)(size_t, int*);
};

using F32Mean = OpMean<float, float, float>;
using F32Sum = OpSumF<float, float, float>;
using F32Diffuse = OpDiffuse<float, float, float>;

#define STC_T2(OPV, OPT, KIND)                                                                            \
    Tb2Entry{OPV, KIND, tb2_launch<OPT, Shape<KIND, 1, 2>, 4>, tb2_launch<OPT, Shape<KIND, 1, 2>, 8>,      \
             tb2_occupancy<OPT, Shape<KIND, 1, 2>, 4>}
static const Tb2Entry kTb2Table[] = {
    STC_T2(OPV_MEAN, F32Mean, STC_SHAPE_WINDOW),
    STC_T2(OPV_SUM, F32Sum, STC_SHAPE_WINDOW),
    STC_T2(OPV_MEAN, F32Mean, STC_SHAPE_MOORE),
    STC_T2(OPV_SUM, F32Sum, STC_SHAPE_MOORE),
    STC_T2(OPV_MEAN, F32Mean, STC_SHAPE_VONNEUMANN),
    STC_T2(OPV_SUM, F32Sum, STC_SHAPE_VONNEUMANN),
    STC_T2(OPV_DIFFUSE, F32Diffuse, STC_SHAPE_VONNEUMANN),
};
#undef STC_T2

static const Tb2Entry* tb2_find(const stc_grid* a, const stc_stencil* st, const stc_op* op) {
    if (a->dtype != STC_F32 || a->ndims != 2 || st->ndims != 2 || st->radius != 1) return nullptr;
    const int opv = op->code == STC_OP_DIFFUSE ? OPV_DIFFUSE : op->code == STC_OP_MEAN ? OPV_MEAN
                    : op->code == STC_OP_SUM ? OPV_SUM : -1;
    for (const Tb2Entry& e : kTb2Table)
        if (e.opv == opv && table_matches_shape(e.shape, 1, 2, st->offsets, st->len)) return &e;
    return nullptr;
}

bool tb2d_applies(const stc_grid* a, const stc_stencil* st, const stc_op* op, const stc_bc* bc) {
    if (!(bc->boundary == STC_WRAP || bc->boundary == STC_REMOVE)) return false;
    return tb2_find(a, st, op) != nullptr;
}

// Levels per pass: 8 (on 8192^2 x 100 Float32 8 levels measured 1007 against 910 Gcell/s for 4 on
// VonNeumann(1) diffusion, 671 against 662 on Window(1) mean before the staged-range test); STC_TB2_K = 4
// overrides, a tuning knob.
static int tb2_levels() {
    const char* e = getenv("STC_TB2_K");
    return (e && atoi(e) == 4) ? 4 : 8;
}

int tb2d_try_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op, const stc_bc* bc,
                   int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx, int64_t* done) {
    *done = 0;
    const char* env = getenv("STC_TBLOCK");
    if (env && env[0] == '0') return STC_OK;
    if (nsteps < 2 || !tb2d_applies(a, st, op, bc)) return STC_OK;
    const Tb2Entry* ent = tb2_find(a, st, op);
    const int K = tb2_levels();
    // Blocked passes take P K steps and the rest (at least one) run as per-step maps, so the pair ends
    // with states n - 1 and n.  A pass advances K (even) steps but switches the parents once, so P is
    // even: then state n lands in the parent the reference's loop leaves it in (b after an odd number of
    // steps, a after an even number).
    int64_t passes = (nsteps - 1) / K;
    passes -= passes & 1;
    const int64_t blocked = passes * K;
    if (blocked < K) return STC_OK;
    const bool halo = bc->padding != STC_CONDITIONAL;
    const int64_t n0 = a->size[0] - (halo ? 2 : 0), n1 = a->size[1] - (halo ? 2 : 0);
    if (n0 < 1 || n1 < 1 || n0 > (1 << 30) || n1 > (1 << 30)) return STC_OK;
    TB2Params p;
    memset(&p, 0, sizeof(p));
    p.BY = 64;
    p.TX = kT2BX - 2 * K;
    p.TY = p.BY - 2 * K;
    const size_t smem = (size_t)2 * kT2BX * p.BY * sizeof(float);
    if ((int64_t)smem > ctx->max_smem_optin) return STC_OK;
    p.n0 = (int32_t)n0;
    p.n1 = (int32_t)n1;
    p.ntx = (int32_t)((n0 + p.TX - 1) / p.TX);
    const int64_t nty = (n1 + p.TY - 1) / p.TY;
    if ((int64_t)p.ntx * nty >= (1ll << 31)) return STC_OK;
    p.ntiles = (int32_t)(p.ntx * nty);
    p.remove = bc->boundary == STC_REMOVE;
    p.status = status_slot(ctx, stream).dev;
    p.padf = (float)bc->padval;
    p.L = st->len;
    p.alpha = op->alpha;
    p.rcp_f = (float)(1.0 / (double)st->len);
    p.fastdiv_f = op->code == STC_OP_MEAN ? (int)fastdiv_f_exact(st->len) : 0;
    p.Lf = (float)st->len;
    p.Ld = (double)st->len;
    p.alpha_f = (float)op->alpha;
    int per_sm = 0;
    cudaError_t e = ent->occ4(smem, &per_sm);
    if (e != cudaSuccess) return cuda_fail(e);
    if (per_sm < 1) return STC_OK;
    const int grid = (int)std::min<int64_t>(p.ntiles, (int64_t)per_sm * ctx->num_sms);
    Tb2Launch fn = K == 8 ? ent->fn8 : ent->fn4;
    const stc_grid* par[2] = {a, b};
    int cur = *src_is_b;
    for (int64_t step = 0; step < blocked; step += K) {
        const stc_grid* sg = par[cur];
        const stc_grid* dg = par[1 - cur];
        const int64_t so = halo ? 1 + sg->stride[1] : 0, dof = halo ? 1 + dg->stride[1] : 0;
        p.src = (const float*)sg->data + so;
        p.dst = (float*)dg->data + dof;
        p.sstr = sg->stride[1];
        p.dstr = dg->stride[1];
        // 16-byte staging when every box row starts on a 16-byte boundary (box columns start at
        // multiples of TX = 128 - 2K minus K: multiples of 4 for K = 4 and 8)
        p.vec_ok = ((uintptr_t)p.src % 16 == 0) && (p.sstr % 4 == 0) && (K % 4 == 0);
        void* prof = prof_begin(stream);
        e = fn(p, grid, smem, stream);
        prof_end(prof, stream, "tblock2d", 8.0 * n0 * n1 * K, (double)n0 * n1 * K);
        if (e != cudaSuccess) return cuda_fail(e);
        cur = 1 - cur;
    }
    *src_is_b = cur;
    *done = blocked;
    return STC_OK;
}

}  // namespace stc
