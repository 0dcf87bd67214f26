// life.cu — K3: bit-packed, temporally blocked outer-totalistic Moore(1) cellular automata.
//
// Replaces the loop  A = mapstencil!(rule, A::SwitchingStencilArray)  (src/gatherstencil.jl:77-83,
// src/array.jl:610-611) for 2D Moore(1) rules on UInt8 / Bool / Int32 / Int64 grids.
//
// Layout: the logical grid is packed 32 cells per 32-bit word along the contiguous axis (bit j of
// word w is cell 32w + j), rows stacked along axis 1.  A launch advances every row band by up to k
// generations: each CTA holds full rows (the x-wrap happens inside shared memory) for its band plus
// k halo rows above and below (y-wrap or zero rows from global), steps them k times in a shared
// ping-pong pair — the valid band shrinks by one row per generation — and writes the band back.
// One HBM/L2 round trip per k generations instead of per generation.
//
// Per word, each row's 3-cell sum (2 bits, from funnel shifts of its (w-1, w, w+1) words) is formed
// once as the row enters a rolling three-row window; a carry-save adder adds the three rows' sums into
// the 4-bit 3x3 total and the rule is evaluated bitwise on it (neighbours = total - centre).
// The neighbour count is the count of nonzero neighbours, exactly what the LIFE op counts, so the
// result is bit-identical to the per-cell gather for any input values.
#include <algorithm>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "life.h"
#include "profile.h"

namespace stc {

constexpr int kLifeThreads = 512;

struct Count4 { uint32_t b0, b1, b2, b3; };

__device__ __forceinline__ void full_add(uint32_t a, uint32_t b, uint32_t c, uint32_t& s, uint32_t& cy) {
    const uint32_t t = a ^ b;
    s = t ^ c;
    cy = (a & b) | (t & c);
}

// 3-cell horizontal sum of a row around every bit: (a, b) with L + C + R = a + 2b
struct Sum3 { uint32_t a, b; };
__device__ __forceinline__ Sum3 row_sum3(uint32_t wl, uint32_t c, uint32_t wr) {
    const uint32_t L = __funnelshift_l(wl, c, 1), R = __funnelshift_r(c, wr, 1);
    Sum3 s;
    s.a = L ^ c ^ R;
    s.b = (L & c) | (R & (L ^ c));
    return s;
}

// 4-bit total of the 3x3 block (centre included) from three rows' 3-cell sums
__device__ __forceinline__ Count4 total9(const Sum3& u, const Sum3& c, const Sum3& d) {
    Count4 t;
    uint32_t k0, x1, k1;
    full_add(u.a, c.a, d.a, t.b0, k0);     // weight 1 and its carry (weight 2)
    full_add(u.b, c.b, d.b, x1, k1);       // weight 2 and its carry (weight 4)
    t.b1 = x1 ^ k0;
    const uint32_t k2 = x1 & k0;           // weight 4
    t.b2 = k1 ^ k2;
    t.b3 = k1 & k2;                         // weight 8
    return t;
}

// next state from the 3x3 total (neighbour count n = total - centre)
template <bool CONWAY>
__device__ __forceinline__ uint32_t rule_from_total(const Count4& t, uint32_t c, uint32_t birth, uint32_t survive) {
    if constexpr (CONWAY) {
        // B3/S23: n == 3 (total 3 when dead, 4 when alive) or alive with n == 2 (total 3)
        const uint32_t is3 = t.b0 & t.b1 & ~t.b2 & ~t.b3;
        const uint32_t is4 = ~t.b0 & ~t.b1 & t.b2 & ~t.b3;
        return is3 | (c & is4);
    } else {
        uint32_t out = 0;
#pragma unroll
        for (int v = 0; v <= 9; ++v) {
            const uint32_t m = ((v & 1) ? t.b0 : ~t.b0) & ((v & 2) ? t.b1 : ~t.b1) & ((v & 4) ? t.b2 : ~t.b2) &
                               ((v & 8) ? t.b3 : ~t.b3);
            if (v <= 8 && ((birth >> v) & 1u)) out |= m & ~c;             // dead: n = total
            if (v >= 1 && ((survive >> (v - 1)) & 1u)) out |= m & c;     // alive: n = total - 1
        }
        return out;
    }
}

struct LifeParams {
    const uint32_t* in;
    uint32_t* out;
    int W;          // words per row
    int n1;         // rows
    int TB;         // band rows written back per CTA
    int k;          // generations this launch
    int wrap;       // 1: Wrap, 0: Remove(0)
    uint32_t birth, survive;
};

// one column's rolling window: the 3-cell sums of the rows above and at the current row, and the
// current row's own word
struct ColState { Sum3 su, sc; uint32_t c; };

template <bool WRAP>
__device__ __forceinline__ Sum3 load_sum3(const uint32_t* row, int w, int wl, int wr, int W) {
    const uint32_t C = row[w];
    const uint32_t L = (!WRAP && w == 0) ? 0u : row[wl];
    const uint32_t R = (!WRAP && w == W - 1) ? 0u : row[wr];
    return row_sum3(L, C, R);
}

template <bool CONWAY, bool WRAP>
__global__ void __launch_bounds__(kLifeThreads) life_block_kernel(const LifeParams p) {
    extern __shared__ __align__(16) uint32_t lsm[];
    const int W = p.W, k = p.k;
    const int rows = p.TB + 2 * k;
    uint32_t* buf0 = lsm;
    uint32_t* buf1 = lsm + (size_t)rows * W;
    const int y0 = blockIdx.x * p.TB;
    // load the band plus k halo rows
    for (int i = threadIdx.x; i < rows * W; i += blockDim.x) {
        const int r = i / W, w = i - r * W;
        int gy = y0 - k + r;
        uint32_t v = 0;
        if (WRAP) {
            gy %= p.n1;
            if (gy < 0) gy += p.n1;
            v = p.in[(size_t)gy * W + w];
        } else if (gy >= 0 && gy < p.n1) {
            v = p.in[(size_t)gy * W + w];
        }
        buf0[i] = v;
    }
    __syncthreads();
    // Thread -> (column pair, strip).  Each thread carries two independent columns (w and w + W/2
    // when W is even) through its strip of rows, so the two adder networks interleave.  Strips split
    // the valid row range of each generation.
    const int cols = (W % 2 == 0) ? 2 : 1;
    const int Wc = W / cols;
    const int strips = max(1, (int)blockDim.x / Wc);
    for (int g = 0; g < k; ++g) {
        const uint32_t* src = (g & 1) ? buf1 : buf0;
        uint32_t* dst = (g & 1) ? buf0 : buf1;
        const int lo = g + 1, hi = rows - g - 1;   // rows computable from the valid rows of src
        const int nr = hi - lo;
        for (int item = threadIdx.x; item < Wc * strips; item += blockDim.x) {
            const int cb = item % Wc, s = item / Wc;
            const int ra = lo + (nr * s) / strips, rb = lo + (nr * (s + 1)) / strips;
            if (ra >= rb) continue;
            int w[2], wl[2], wr[2];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                w[j] = cb + j * Wc;
                wl[j] = w[j] == 0 ? W - 1 : w[j] - 1;
                wr[j] = w[j] == W - 1 ? 0 : w[j] + 1;
            }
            ColState st[2];
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                if (j >= cols) break;
                st[j].su = load_sum3<WRAP>(src + (ra - 1) * W, w[j], wl[j], wr[j], W);
                st[j].sc = load_sum3<WRAP>(src + ra * W, w[j], wl[j], wr[j], W);
                st[j].c = src[ra * W + w[j]];
            }
            for (int r = ra; r < rb; ++r) {
                const uint32_t* nrow = src + (r + 1) * W;
                bool dead_row = false;
                if (!WRAP) {
                    const int gy = y0 - k + r;
                    dead_row = gy < 0 || gy >= p.n1;   // rows outside the grid stay dead
                }
#pragma unroll
                for (int j = 0; j < 2; ++j) {
                    if (j >= cols) break;
                    const Sum3 sd = load_sum3<WRAP>(nrow, w[j], wl[j], wr[j], W);
                    const uint32_t cd = nrow[w[j]];
                    uint32_t nx = rule_from_total<CONWAY>(total9(st[j].su, st[j].sc, sd), st[j].c, p.birth, p.survive);
                    if (dead_row) nx = 0u;
                    dst[r * W + w[j]] = nx;
                    st[j].su = st[j].sc;
                    st[j].sc = sd;
                    st[j].c = cd;
                }
            }
        }
        __syncthreads();
    }
    const uint32_t* fin = (k & 1) ? buf1 : buf0;
    for (int i = threadIdx.x; i < p.TB * W; i += blockDim.x) {
        const int r = i / W, w = i - r * W;
        const int gy = y0 + r;
        if (gy < p.n1) p.out[(size_t)gy * W + w] = fin[(size_t)(r + k) * W + w];
    }
}

// launch one k-generation pass (both entry points use this)
static cudaError_t life_launch(const LifeParams& lp, bool conway, int grid, size_t smem, cudaStream_t s) {
#define STC_LIFE_LAUNCH(C, WR)                                                                       \
    {                                                                                                \
        cudaError_t e = cudaFuncSetAttribute(life_block_kernel<C, WR>,                                \
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); \
        if (e != cudaSuccess) return e;                                                              \
        life_block_kernel<C, WR><<<grid, kLifeThreads, smem, s>>>(lp);                               \
        return cudaGetLastError();                                                                   \
    }
    if (conway && lp.wrap) STC_LIFE_LAUNCH(true, true)
    if (conway) STC_LIFE_LAUNCH(true, false)
    if (lp.wrap) STC_LIFE_LAUNCH(false, true)
    STC_LIFE_LAUNCH(false, false)
#undef STC_LIFE_LAUNCH
}

// ------------------------------------------------------------------ pack / unpack
struct PackParams {
    const void* base;   // parent base
    int64_t org;        // parent offset of logical (0, 0)
    int64_t sy;         // parent row stride (elements)
    int dt;
    int W, n1;
    uint32_t* P;
};

template <class T>
__global__ void life_pack_kernel(const PackParams p) {
    const T* base = (const T*)p.base;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t groups = (int64_t)p.n1 * ((p.W + 31) / 32);
    for (int64_t gi = warp; gi < groups; gi += nwarps) {
        const int gpr = (p.W + 31) / 32;
        const int y = (int)(gi / gpr), w0 = (int)(gi % gpr) * 32;
        const T* row = base + p.org + (int64_t)y * p.sy;
        uint32_t mine = 0;
        const int nw = min(32, p.W - w0);
        for (int i = 0; i < nw; ++i) {
            const uint32_t b = __ballot_sync(0xffffffffu, row[(int64_t)(w0 + i) * 32 + lane] != (T)0);
            if (lane == i) mine = b;
        }
        if (lane < nw) p.P[(size_t)y * p.W + w0 + lane] = mine;
    }
}

template <class T>
__global__ void life_unpack_kernel(const PackParams p) {
    T* base = (T*)p.base;
    const int lane = threadIdx.x & 31;
    const int64_t warp = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    const int64_t groups = (int64_t)p.n1 * ((p.W + 31) / 32);
    for (int64_t gi = warp; gi < groups; gi += nwarps) {
        const int gpr = (p.W + 31) / 32;
        const int y = (int)(gi / gpr), w0 = (int)(gi % gpr) * 32;
        T* row = base + p.org + (int64_t)y * p.sy;
        const int nw = min(32, p.W - w0);
        const uint32_t mine = lane < nw ? p.P[(size_t)y * p.W + w0 + lane] : 0u;
        for (int i = 0; i < nw; ++i) {
            const uint32_t word = __shfl_sync(0xffffffffu, mine, i);
            row[(int64_t)(w0 + i) * 32 + lane] = (T)((word >> lane) & 1u);
        }
    }
}

static int launch_pack(bool pack, const stc_grid* g, int64_t org, int W, int n1, uint32_t* P, cudaStream_t s,
                       int num_sms) {
    PackParams p{};
    p.base = g->data;
    p.org = org;
    p.sy = g->stride[1];
    p.dt = g->dtype;
    p.W = W;
    p.n1 = n1;
    p.P = P;
    const int64_t groups = (int64_t)n1 * ((W + 31) / 32);
    int blocks = (int)std::min<int64_t>((groups * 32 + 255) / 256, (int64_t)num_sms * 8);
    blocks = std::max(blocks, 1);
    void* prof = prof_begin(s);
#define STC_PACK_CASE(DT, T)                                                                       \
    case DT:                                                                                       \
        if (pack) life_pack_kernel<T><<<blocks, 256, 0, s>>>(p); else life_unpack_kernel<T><<<blocks, 256, 0, s>>>(p); \
        break;
    switch (g->dtype) {
        STC_PACK_CASE(STC_U8, uint8_t)
        STC_PACK_CASE(STC_BOOL, uint8_t)
        STC_PACK_CASE(STC_I32, int32_t)
        STC_PACK_CASE(STC_I64, int64_t)
    default: return STC_ERR_UNSUPPORTED;
    }
#undef STC_PACK_CASE
    prof_end(prof, s, pack ? "life_pack" : "life_unpack", (double)W * 32 * n1 * (dtype_size(g->dtype) + 0.125),
             (double)W * 32 * n1);
    return cuda_fail(cudaGetLastError());
}

// ------------------------------------------------------------------ host
static bool is_moore1_2d(const stc_stencil* st) {
    if (st->ndims != 2 || st->len != 8 || st->radius != 1) return false;
    static const int want[16] = {-1, -1, 0, -1, 1, -1, -1, 0, 1, 0, -1, 1, 0, 1, 1, 1};
    for (int i = 0; i < 16; ++i)
        if (st->offsets[i] != want[i]) return false;
    return true;
}

// Band rows and generations per launch for a grid of W words x n1 rows: one band per SM when the
// grid is tall enough (the kernel is ALU-bound, so every SM should hold one band), at most 16
// generations per launch, and whatever fits in shared memory.
void life_plan(int W, int n1, int64_t steps_left, int smem_cap, int num_sms, int* TB, int* k) {
    int kk = (int)std::min<int64_t>(steps_left, 16);
    int tb = std::max(8, (n1 + num_sms - 1) / num_sms);
    while (kk > 1 && (int64_t)2 * (tb + 2 * kk) * W * 4 > smem_cap) --kk;
    while (tb > 1 && (int64_t)2 * (tb + 2 * kk) * W * 4 > smem_cap) --tb;
    *TB = tb;
    *k = kk;
}

int life_try_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op, const stc_bc* bc,
                   int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx, int64_t* done) {
    *done = 0;
    if (nsteps < 1 || op->code != STC_OP_LIFE || a->ndims != 2 || !is_moore1_2d(st)) return STC_OK;
    if (!(a->dtype == STC_U8 || a->dtype == STC_BOOL || a->dtype == STC_I32 || a->dtype == STC_I64)) return STC_OK;
    const bool halo = bc->padding != STC_CONDITIONAL;
    const bool wrap = bc->boundary == STC_WRAP;
    const bool remove0 = bc->boundary == STC_REMOVE && bc->padval_int == 0;
    if (!wrap && !remove0) return STC_OK;   // Reflect / Use / nonzero padval take the per-step kernel
    const int64_t n0 = a->size[0] - (halo ? 2 : 0), n1 = a->size[1] - (halo ? 2 : 0);
    if (n0 < 32 || n0 % 32 != 0 || n1 < 1 || n0 / 32 > 512 || n1 > (1 << 30)) return STC_OK;
    const int W = (int)(n0 / 32);
    const int smem_cap = ctx->max_smem_optin - 1024;
    int TB, k;
    life_plan(W, (int)n1, nsteps, smem_cap, ctx->num_sms, &TB, &k);
    if ((int64_t)2 * (TB + 2 * k) * W * 4 > smem_cap) return STC_OK;

    const size_t words = (size_t)W * n1;
    uint32_t* P = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&P, 2 * words * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return cuda_fail(e);
    uint32_t* Pbuf[2] = {P, P + words};
    const int64_t org_a = halo ? 1 + a->stride[1] : 0, org_b = halo ? 1 + b->stride[1] : 0;
    int rc = launch_pack(true, a, org_a, W, (int)n1, Pbuf[0], stream, ctx->num_sms);
    if (rc) { cudaFreeAsync(P, stream); return rc; }

    LifeParams lp{};
    lp.W = W;
    lp.n1 = (int)n1;
    lp.wrap = wrap;
    lp.birth = op->birth_mask;
    lp.survive = op->survive_mask;
    const bool conway = op->birth_mask == (1u << 3) && op->survive_mask == ((1u << 2) | (1u << 3));
    int cur = 0;
    int64_t left = nsteps;
    while (left > 0) {
        // the last generation runs alone so both packed buffers hold the last two states
        const int64_t budget = left > 1 ? left - 1 : 1;
        life_plan(W, (int)n1, budget, smem_cap, ctx->num_sms, &TB, &k);
        lp.in = Pbuf[cur];
        lp.out = Pbuf[1 - cur];
        lp.TB = TB;
        lp.k = k;
        const size_t smem = (size_t)2 * (TB + 2 * k) * W * 4;
        const int grid = (int)((n1 + TB - 1) / TB);
        void* prof = prof_begin(stream);
        e = life_launch(lp, conway, grid, smem, stream);
        prof_end(prof, stream, "life_block", 2.0 * n0 * n1 * k, (double)n0 * n1 * k);
        if (e != cudaSuccess) { cudaFreeAsync(P, stream); return cuda_fail(e); }
        cur = 1 - cur;
        left -= k;
    }
    // Pbuf[cur] holds generation nsteps, Pbuf[1-cur] generation nsteps-1 (or the input if nsteps == 1).
    // The reference leaves the result in b after an odd number of steps, in a after an even number.
    const bool res_in_b = (nsteps & 1) != 0;
    const stc_grid* res = res_in_b ? b : a;
    const stc_grid* prev = res_in_b ? a : b;
    rc = launch_pack(false, res, res_in_b ? org_b : org_a, W, (int)n1, Pbuf[cur], stream, ctx->num_sms);
    if (!rc && nsteps > 1) rc = launch_pack(false, prev, res_in_b ? org_a : org_b, W, (int)n1, Pbuf[1 - cur], stream, ctx->num_sms);
    cudaFreeAsync(P, stream);
    if (rc) return rc;
    *src_is_b = res_in_b ? 1 : 0;
    *done = nsteps;
    return STC_OK;
}

}  // namespace stc

// ------------------------------------------------------------------ no-allocation variant
// stc_life_steps_noalloc: the same packed kernels with the two packed copies in a fixed array that
// is part of the library image, for callers that cannot allocate device memory (see the header).
namespace stc {

constexpr int64_t kNoAllocMaxCells = 4096ll * 4096ll;
constexpr int64_t kNoAllocWords = kNoAllocMaxCells / 32;   // one packed copy

// Two packed copies, 4 MiB in total.  In host code this name is only a stand-in for the device
// array; the kernels get its device address from cudaGetSymbolAddress.
static __device__ __align__(256) uint32_t g_noalloc_scratch[2 * kNoAllocWords];

static std::mutex g_noalloc_mu;
static uint32_t* g_noalloc_ptr[64] = {nullptr};

static int noalloc_scratch(int dev, uint32_t** out) {
    if (dev < 0 || dev >= 64) return STC_ERR_NO_DEVICE;
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void* ptr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);   // current device is `dev`
        if (e != cudaSuccess) return cuda_fail(e);
        g_noalloc_ptr[dev] = (uint32_t*)ptr;
    }
    *out = g_noalloc_ptr[dev];
    return STC_OK;
}

template <class T>
static void noalloc_pack(bool pack, const PackParams& p, int blocks, cudaStream_t s) {
    if (pack) life_pack_kernel<T><<<blocks, 256, 0, s>>>(p);
    else life_unpack_kernel<T><<<blocks, 256, 0, s>>>(p);
}

static int noalloc_pack_launch(bool pack, const stc_grid* g, int64_t org, int W, int n1, uint32_t* P,
                               cudaStream_t s, int num_sms) {
    PackParams p{};
    p.base = g->data;
    p.org = org;
    p.sy = g->stride[1];
    p.dt = g->dtype;
    p.W = W;
    p.n1 = n1;
    p.P = P;
    const int64_t groups = (int64_t)n1 * ((W + 31) / 32);
    const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((groups * 32 + 255) / 256, (int64_t)num_sms * 8));
    switch (g->dtype) {
    case STC_U8: case STC_BOOL: noalloc_pack<uint8_t>(pack, p, blocks, s); break;
    case STC_I32: noalloc_pack<int32_t>(pack, p, blocks, s); break;
    case STC_I64: noalloc_pack<int64_t>(pack, p, blocks, s); break;
    default: return STC_ERR_UNSUPPORTED;
    }
    return cuda_fail(cudaGetLastError());
}

}  // namespace stc

extern "C" int stc_life_steps_noalloc(const stc_grid* a, const stc_grid* b, const stc_stencil* st,
                                      const stc_op* op, const stc_bc* bc, int64_t nsteps, int32_t* out_src_is_b,
                                      void* stream) {
    using namespace stc;
    if (nsteps < 0) return STC_ERR_INVALID;
    int rc = validate_map(a, b, 1, st, op, bc);
    if (rc) return rc;
    for (int d = 0; d < a->ndims; ++d)
        if (a->size[d] != b->size[d] || a->dtype != b->dtype) return STC_ERR_SIZE_MISMATCH;
    if (op->code != STC_OP_LIFE || a->ndims != 2 || !is_moore1_2d(st)) return STC_ERR_UNSUPPORTED;
    if (!(a->dtype == STC_U8 || a->dtype == STC_BOOL || a->dtype == STC_I32 || a->dtype == STC_I64))
        return STC_ERR_UNSUPPORTED;
    const bool halo = bc->padding != STC_CONDITIONAL;
    const bool wrap = bc->boundary == STC_WRAP;
    const bool remove0 = bc->boundary == STC_REMOVE && bc->padval_int == 0;
    if (!wrap && !remove0) return STC_ERR_UNSUPPORTED;
    const int64_t n0 = a->size[0] - (halo ? 2 : 0), n1 = a->size[1] - (halo ? 2 : 0);
    if (n0 < 32 || n0 % 32 != 0 || n1 < 1) return STC_ERR_UNSUPPORTED;
    if (n0 * n1 > kNoAllocMaxCells) return STC_ERR_TOO_LARGE;
    if (nsteps > 0 && a->data == b->data) return STC_ERR_INVALID;
    if (nsteps == 0) {
        if (out_src_is_b) *out_src_is_b = 0;
        return STC_OK;
    }
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) { cuda_fail(e); return STC_ERR_NO_DEVICE; }
    int num_sms = 0, smem_optin = 0;
    if ((e = cudaDeviceGetAttribute(&num_sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return cuda_fail(e);
    if ((e = cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess)
        return cuda_fail(e);
    uint32_t* P = nullptr;
    if ((rc = noalloc_scratch(dev, &P))) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    const int W = (int)(n0 / 32);
    const int smem_cap = smem_optin - 1024;
    int TB, k;
    life_plan(W, (int)n1, nsteps, smem_cap, num_sms, &TB, &k);
    if ((int64_t)2 * (TB + 2 * k) * W * 4 > smem_cap) return STC_ERR_UNSUPPORTED;
    uint32_t* Pbuf[2] = {P, P + kNoAllocWords};
    const int64_t org_a = halo ? 1 + a->stride[1] : 0, org_b = halo ? 1 + b->stride[1] : 0;
    if ((rc = noalloc_pack_launch(true, a, org_a, W, (int)n1, Pbuf[0], s, num_sms))) return rc;
    LifeParams lp{};
    lp.W = W;
    lp.n1 = (int)n1;
    lp.wrap = wrap;
    lp.birth = op->birth_mask;
    lp.survive = op->survive_mask;
    const bool conway = op->birth_mask == (1u << 3) && op->survive_mask == ((1u << 2) | (1u << 3));
    int cur = 0;
    int64_t left = nsteps;
    while (left > 0) {
        const int64_t budget = left > 1 ? left - 1 : 1;
        life_plan(W, (int)n1, budget, smem_cap, num_sms, &TB, &k);
        lp.in = Pbuf[cur];
        lp.out = Pbuf[1 - cur];
        lp.TB = TB;
        lp.k = k;
        const size_t smem = (size_t)2 * (TB + 2 * k) * W * 4;
        const int grid = (int)((n1 + TB - 1) / TB);
        if ((e = life_launch(lp, conway, grid, smem, s)) != cudaSuccess) return cuda_fail(e);
        cur = 1 - cur;
        left -= k;
    }
    const bool res_in_b = (nsteps & 1) != 0;
    const stc_grid* res = res_in_b ? b : a;
    const stc_grid* prev = res_in_b ? a : b;
    if ((rc = noalloc_pack_launch(false, res, res_in_b ? org_b : org_a, W, (int)n1, Pbuf[cur], s, num_sms))) return rc;
    if (nsteps > 1 &&
        (rc = noalloc_pack_launch(false, prev, res_in_b ? org_a : org_b, W, (int)n1, Pbuf[1 - cur], s, num_sms)))
        return rc;
    if (out_src_is_b) *out_src_is_b = res_in_b ? 1 : 0;
    return cuda_fail(cudaStreamSynchronize(s));
}
