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
#include <cstdlib>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "life.h"
#include "profile.h"

namespace stc {

constexpr int kLifeMaxThreads = 1024;

// CTA size of the Life kernels: 512 threads (STC_LIFE_THREADS = 1024 overrides, a tuning knob)
static int life_threads() {
    const char* e = getenv("STC_LIFE_THREADS");
    return (e && atoi(e) == 1024) ? 1024 : 512;
}

__device__ __forceinline__ void full_add(uint32_t a, uint32_t b, uint32_t c, uint32_t& s, uint32_t& cy) {
    const uint32_t t = a ^ b;
    s = t ^ c;
    cy = (a & b) | (t & c);
}

// One source row seen from one column word: its 3-cell sums around every bit (a3 + 2 b3 = L + C + R,
// used when the row is above or below the output row), its 2-cell sums (a2 + 2 b2 = L + R, used when
// it is the output's own row) and the centre word itself.
struct RowV { uint32_t a3, b3, a2, b2, c; };

__device__ __forceinline__ RowV row_v(uint32_t wl, uint32_t c, uint32_t wr) {
    const uint32_t L = __funnelshift_l(wl, c, 1), R = __funnelshift_r(c, wr, 1);
    RowV v;
    v.a3 = L ^ c ^ R;
    v.b3 = (L & c) | (R & (L ^ c));
    v.a2 = L ^ R;
    v.b2 = L & R;
    v.c = c;
    return v;
}

// next state of the middle row m from the neighbour count n = sum3(u) + sum2(m) + sum3(d), 0..8, held
// as bit planes n0..n3 (B3/S23 uses the 3x3 total instead)
template <bool CONWAY>
__device__ __forceinline__ uint32_t next_state(const RowV& u, const RowV& m, const RowV& d, uint32_t birth,
                                               uint32_t survive) {
    if constexpr (CONWAY) {
        // B3/S23 from the 3x3 total t = n + centre (0..9): alive next iff t == 3, or t == 4 and alive.
        // Only t's low three bits are formed: t in {3, 4} is exactly (t0^t2) & (t1^t2) (8 and 9 fail
        // it), and t2 tells the two apart.
        uint32_t t0, k0, x1, k1;
        full_add(u.a3, m.a3, d.a3, t0, k0);
        full_add(u.b3, m.b3, d.b3, x1, k1);
        const uint32_t t1 = x1 ^ k0;
        const uint32_t t2 = k1 ^ (x1 & k0);
        return ((t0 ^ t2) & (t1 ^ t2)) & (~t2 | m.c);
    } else {
        uint32_t n0, k0, x1, k1;
        full_add(u.a3, m.a2, d.a3, n0, k0);    // weight 1 and its carry (weight 2)
        full_add(u.b3, m.b2, d.b3, x1, k1);    // weight 2 and its carry (weight 4)
        const uint32_t n1 = x1 ^ k0;
        const uint32_t n2 = k1 ^ (x1 & k0);
        const uint32_t n3 = k1 & x1 & k0;
        uint32_t out = 0;
#pragma unroll
        for (int v = 0; v <= 8; ++v) {
            const uint32_t eq = ((v & 1) ? n0 : ~n0) & ((v & 2) ? n1 : ~n1) & ((v & 4) ? n2 : ~n2) &
                                ((v & 8) ? n3 : ~n3);
            if ((birth >> v) & 1u) out |= eq & ~m.c;
            if ((survive >> v) & 1u) out |= eq & m.c;
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

// A thread's fixed share of a band: one column w (or two, w and w + W/2, for narrow rows) and strip s
// of `strips` row strips.  One column per thread means fewer, longer strips, so the two rows each
// strip reads before its first output are a smaller share of the work; the unrolled row walk gives
// the thread its independent instructions.  Computed once per kernel.
struct LifeLane {
    int cols;            // 0 (idle thread), 1 or 2
    int w[2], wl[2], wr[2];
    bool ledge[2], redge[2];
    int s, strips;
    float inv_strips;
};

__device__ __forceinline__ LifeLane life_lane(int W) {
    LifeLane L;
    const int cols = (W % 2 == 0 && W < 64) ? 2 : 1;
    const int Wc = W / cols;
    L.strips = max(1, (int)blockDim.x / Wc);
    L.inv_strips = 1.0f / (float)L.strips;
    const int item = threadIdx.x;
    L.cols = item < Wc * L.strips ? cols : 0;
    const int cb = item % Wc;
    L.s = item / Wc;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        L.w[j] = cb + j * Wc;
        L.ledge[j] = L.w[j] == 0;
        L.redge[j] = L.w[j] == W - 1;
        L.wl[j] = L.ledge[j] ? W - 1 : L.w[j] - 1;
        L.wr[j] = L.redge[j] ? 0 : L.w[j] + 1;
    }
    return L;
}

// Rows [ra, rb) of one strip for NC columns: source row q is read through per-column pointers to
// its (w-1, w, w+1) words, each row's sums are formed once as it enters a three-row window, and the
// row walk is unrolled by three with the window's roles rotating, so nothing is copied between
// registers.  Remove(0) (WRAP false): words beyond the x edges read as zero, and rows outside the grid
// stay dead.
template <bool CONWAY, bool WRAP, int WT, int NC>
__device__ __forceinline__ void life_strip(const LifeLane& L, const uint32_t* src, uint32_t* dst, int Wrt, int ra,
                                           int rb, int gy_first, int n1, uint32_t birth, uint32_t survive) {
    const int W = WT > 0 ? WT : Wrt;
    const uint32_t *pl[NC], *pc[NC], *pr[NC];
    uint32_t* pd[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        pl[j] = src + (size_t)(ra - 1) * W + L.wl[j];
        pc[j] = src + (size_t)(ra - 1) * W + L.w[j];
        pr[j] = src + (size_t)(ra - 1) * W + L.wr[j];
        pd[j] = dst + (size_t)ra * W + L.w[j];
    }
    // row (ra - 1 + q) of column j
    auto load = [&](int j, int q) -> RowV {
        const uint32_t c = pc[j][q * W];
        const uint32_t l = (!WRAP && L.ledge[j]) ? 0u : pl[j][q * W];
        const uint32_t r = (!WRAP && L.redge[j]) ? 0u : pr[j][q * W];
        return row_v(l, c, r);
    };
    // output row (ra + q) from the window (u, m, d)
    auto emit = [&](int j, int q, int r, const RowV& u, const RowV& m, const RowV& d) {
        uint32_t nx = next_state<CONWAY>(u, m, d, birth, survive);
        if (!WRAP) {
            const int gy = gy_first + r;
            if (gy < 0 || gy >= n1) nx = 0u;   // rows outside the grid stay dead
        }
        pd[j][q * W] = nx;
    };
    RowV v0[NC], v1[NC], v2[NC];
#pragma unroll
    for (int j = 0; j < NC; ++j) {
        v0[j] = load(j, 0);
        v1[j] = load(j, 1);
    }
    int r = ra;
    // invariant: v0 = row r-1, v1 = row r; pointers at row r-1 (sources) and row r (destination)
    for (; r + 3 <= rb; r += 3) {
#pragma unroll
        for (int j = 0; j < NC; ++j) v2[j] = load(j, 2);
#pragma unroll
        for (int j = 0; j < NC; ++j) emit(j, 0, r, v0[j], v1[j], v2[j]);
#pragma unroll
        for (int j = 0; j < NC; ++j) v0[j] = load(j, 3);
#pragma unroll
        for (int j = 0; j < NC; ++j) emit(j, 1, r + 1, v1[j], v2[j], v0[j]);
#pragma unroll
        for (int j = 0; j < NC; ++j) v1[j] = load(j, 4);
#pragma unroll
        for (int j = 0; j < NC; ++j) emit(j, 2, r + 2, v2[j], v0[j], v1[j]);
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            pl[j] += 3 * W;
            pc[j] += 3 * W;
            pr[j] += 3 * W;
            pd[j] += 3 * W;
        }
    }
    if (r < rb) {
#pragma unroll
        for (int j = 0; j < NC; ++j) {
            v2[j] = load(j, 2);
            emit(j, 0, r, v0[j], v1[j], v2[j]);
        }
        if (r + 1 < rb) {
#pragma unroll
            for (int j = 0; j < NC; ++j) {
                v0[j] = load(j, 3);
                emit(j, 1, r + 1, v1[j], v2[j], v0[j]);
            }
        }
    }
}

// Advance a band kk generations in the shared ping-pong pair (cur, oth).  cur holds `rows` valid rows
// of W words; row r is global row gy_first + r.  Generation g computes rows [g+1, rows-g-1) (the
// rows whose three source rows are still valid) into the other buffer, split into the lanes' strips.
// Returns the buffer holding the result.  Ends with a barrier.
template <bool CONWAY, bool WRAP, int WT>
__device__ __forceinline__ uint32_t* life_gens(const LifeLane& L, uint32_t* cur, uint32_t* oth, int rows, int W,
                                               int kk, int gy_first, int n1, uint32_t birth, uint32_t survive) {
    for (int g = 0; g < kk; ++g) {
        const int lo = g + 1, hi = rows - g - 1;   // rows computable from the valid rows of cur
        const int nr = hi - lo;
        // strip bounds: the same monotone expression for a strip's end and the next strip's start, so
        // the strips tile [lo, hi) exactly whatever the float rounding
        const int ra = lo + (int)((float)(nr * L.s) * L.inv_strips);
        const int rb = (L.s == L.strips - 1) ? hi : lo + (int)((float)(nr * (L.s + 1)) * L.inv_strips);
        if (ra < rb) {
            if (L.cols == 2) life_strip<CONWAY, WRAP, WT, 2>(L, cur, oth, W, ra, rb, gy_first, n1, birth, survive);
            else if (L.cols == 1) life_strip<CONWAY, WRAP, WT, 1>(L, cur, oth, W, ra, rb, gy_first, n1, birth, survive);
        }
        __syncthreads();
        uint32_t* t = cur;
        cur = oth;
        oth = t;
    }
    return cur;
}

template <bool CONWAY, bool WRAP, int WT>
__global__ void __launch_bounds__(kLifeMaxThreads) life_block_kernel(const LifeParams p) {
    extern __shared__ __align__(16) uint32_t lsm[];
    const int W = WT > 0 ? WT : p.W, k = p.k;
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
    const LifeLane lane = life_lane(W);
    const uint32_t* fin = life_gens<CONWAY, WRAP, WT>(lane, buf0, buf1, rows, W, k, y0 - k, p.n1, p.birth, p.survive);
    for (int i = threadIdx.x; i < p.TB * W; i += blockDim.x) {
        const int r = i / W, w = i - r * W;
        const int gy = y0 + r;
        if (gy < p.n1) p.out[(size_t)gy * W + w] = fin[(size_t)(r + k) * W + w];
    }
}

// ------------------------------------------------------------------ persistent (cooperative) variant
// One launch runs every generation.  CTA b keeps its band (rows [y0, y1), balanced split of n1) in
// shared memory for the whole run, with k ghost rows above and below.  A super-step advances the band
// kk <= k generations; then the CTA publishes its first and last k band rows to an exchange slot in
// global memory, each word as a 64-bit (super-step tag, word) pair written with a single relaxed
// gpu-scope store.  Before the next super-step every thread reloads its share of the neighbours'
// rows until each pair carries the expected tag (bounded) and copies the words in as ghost rows.  No
// fence or flag sits on the critical path: a pair is atomic, so a matching tag means the word is the
// one published for that super-step.  Two slots alternate: a neighbour overwrites a slot only after
// it has read this CTA's following publication, which this CTA makes after reading that slot.
// Every CTA must be resident at once (cooperative launch), and each band holds at least k rows, so
// ghost rows come only from the adjacent bands.
struct LifeCoopParams {
    const uint32_t* in;   // generation 0; receives generation n-1 (n > 1) once neighbours stopped reading it
    uint32_t* prev;       // == in
    uint32_t* last;       // generation n
    uint64_t* xbuf;       // [2 slots][grid][2 (first, last rows)][k][W] tagged words, zero before launch
    int* status;
    int W, n1, k;
    int64_t nsteps;
    uint32_t birth, survive;
};

__device__ __forceinline__ uint64_t ld_relaxed_gpu(const uint64_t* p) {
    uint64_t v;
    asm volatile("ld.relaxed.gpu.global.b64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_relaxed_gpu(uint64_t* p, uint64_t v) {
    asm volatile("st.relaxed.gpu.global.b64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}

// the word of a tagged pair once its tag equals `tag`; false after ~limit SM clocks
__device__ __forceinline__ bool take_tagged(const uint64_t* p, uint32_t tag, uint32_t* out,
                                            long long limit = 4000000000ll) {
    uint64_t v = ld_relaxed_gpu(p);
    if ((uint32_t)(v >> 32) != tag) {
        const long long t0 = clock64();
        do {
            if (clock64() - t0 > limit) return false;
            v = ld_relaxed_gpu(p);
        } while ((uint32_t)(v >> 32) != tag);
    }
    *out = (uint32_t)v;
    return true;
}

template <bool CONWAY, bool WRAP, int WT>
__global__ void __launch_bounds__(kLifeMaxThreads) life_coop_kernel(const LifeCoopParams p) {
    extern __shared__ __align__(16) uint32_t lsm[];
    const int W = WT > 0 ? WT : p.W, k = p.k, G = gridDim.x, b = blockIdx.x;
    const int y0 = (int)(((int64_t)b * p.n1) / G), y1 = (int)(((int64_t)(b + 1) * p.n1) / G);
    const int TB = y1 - y0, rows = TB + 2 * k;
    const int TBmax = (p.n1 + G - 1) / G;
    uint32_t* cur = lsm;
    uint32_t* oth = lsm + (size_t)(TBmax + 2 * k) * W;
    for (int i = threadIdx.x; i < rows * W; i += blockDim.x) {
        const int r = i / W, w = i - r * W;
        int gy = y0 - k + r;
        uint32_t v = 0;
        if (WRAP) {
            gy = gy < 0 ? gy + p.n1 : (gy >= p.n1 ? gy - p.n1 : gy);
            v = p.in[(size_t)gy * W + w];
        } else if (gy >= 0 && gy < p.n1) {
            v = p.in[(size_t)gy * W + w];
        }
        cur[i] = v;
    }
    __syncthreads();
    const int up = b == 0 ? G - 1 : b - 1, dn = b == G - 1 ? 0 : b + 1;
    const bool has_up = WRAP || b > 0, has_dn = WRAP || b < G - 1;
    const size_t slab = (size_t)k * W;                 // one published row block
    const int64_t nmain = p.nsteps - 1;                // generations before the last one
    const LifeLane lane = life_lane(W);
    int64_t gen = 0;
    for (int step = 0;; ++step) {
        const bool final = gen >= nmain;
        const int kk = final ? 1 : (int)min((int64_t)k, nmain - gen);
        if (step > 0) {
            // ghost rows: the neighbours' publication of super-step step-1 (tag step)
            const uint64_t* xs = p.xbuf + (size_t)((step - 1) & 1) * G * 2 * slab;
            const uint64_t* from_up = xs + ((size_t)up * 2 + 1) * slab;   // neighbour's last k rows
            const uint64_t* from_dn = xs + ((size_t)dn * 2 + 0) * slab;   // neighbour's first k rows
            bool ok = true;
            for (int i = threadIdx.x; i < (int)slab; i += blockDim.x) {
                uint32_t u = 0u, d = 0u;
                if (has_up && ok) ok = take_tagged(from_up + i, (uint32_t)step, &u);
                if (has_dn && ok) ok = take_tagged(from_dn + i, (uint32_t)step, &d);
                cur[i] = u;
                cur[(size_t)(k + TB) * W + i] = d;
            }
            if (!__syncthreads_and(ok)) {
                if (threadIdx.x == 0 && p.status) atomicOr(p.status, DEV_ERR_TIMEOUT);
                return;
            }
            if (final && p.nsteps > 1) {
                // generation n-1: every thread has seen both neighbours' publications (so they are past
                // their initial load), and nobody reads `in` any more
                for (int i = threadIdx.x; i < TB * W; i += blockDim.x) p.prev[(size_t)y0 * W + i] = cur[(size_t)k * W + i];
            }
        }
        cur = life_gens<CONWAY, WRAP, WT>(lane, cur, oth, rows, W, kk, y0 - k, p.n1, p.birth, p.survive);
        oth = (cur == lsm) ? lsm + (size_t)(TBmax + 2 * k) * W : lsm;
        gen += kk;
        if (final) {
            for (int i = threadIdx.x; i < TB * W; i += blockDim.x) p.last[(size_t)y0 * W + i] = cur[(size_t)k * W + i];
            return;
        }
        uint64_t* xd = p.xbuf + (size_t)(step & 1) * G * 2 * slab + (size_t)b * 2 * slab;
        const uint64_t tag = (uint64_t)(uint32_t)(step + 1) << 32;
        for (int i = threadIdx.x; i < (int)slab; i += blockDim.x) {
            st_relaxed_gpu(xd + i, tag | cur[(size_t)k * W + i]);            // band rows y0 .. y0+k-1
            st_relaxed_gpu(xd + slab + i, tag | cur[(size_t)TB * W + i]);    // band rows y1-k .. y1-1
        }
    }
}

// Row width specialised at compile time (128 words = 4096 cells); other widths use the run-time path.
constexpr int kLifeWT = 128;

// launch one k-generation pass (both entry points use this)
template <bool C, bool WR, int WT>
static cudaError_t life_launch_t(const LifeParams& lp, int grid, size_t smem, cudaStream_t s) {
    cudaError_t e = cudaFuncSetAttribute(life_block_kernel<C, WR, WT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem);
    if (e != cudaSuccess) return e;
    life_block_kernel<C, WR, WT><<<grid, life_threads(), smem, s>>>(lp);
    return cudaGetLastError();
}

template <int WT>
static cudaError_t life_launch_w(const LifeParams& lp, bool conway, int grid, size_t smem, cudaStream_t s) {
    if (conway && lp.wrap) return life_launch_t<true, true, WT>(lp, grid, smem, s);
    if (conway) return life_launch_t<true, false, WT>(lp, grid, smem, s);
    if (lp.wrap) return life_launch_t<false, true, WT>(lp, grid, smem, s);
    return life_launch_t<false, false, WT>(lp, grid, smem, s);
}

static cudaError_t life_launch(const LifeParams& lp, bool conway, int grid, size_t smem, cudaStream_t s) {
    return lp.W == kLifeWT ? life_launch_w<kLifeWT>(lp, conway, grid, smem, s) : life_launch_w<0>(lp, conway, grid, smem, s);
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
        if (nw == 32) {
            // all 32 loads issued before the first ballot, so the group costs one memory latency
            bool nz[32];
#pragma unroll
            for (int i = 0; i < 32; ++i) nz[i] = row[(int64_t)(w0 + i) * 32 + lane] != (T)0;
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const uint32_t b = __ballot_sync(0xffffffffu, nz[i]);
                if (lane == i) mine = b;
            }
        } else {
            for (int i = 0; i < nw; ++i) {
                const uint32_t b = __ballot_sync(0xffffffffu, row[(int64_t)(w0 + i) * 32 + lane] != (T)0);
                if (lane == i) mine = b;
            }
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
        if (nw == 32) {
#pragma unroll
            for (int i = 0; i < 32; ++i) {
                const uint32_t word = __shfl_sync(0xffffffffu, mine, i);
                row[(int64_t)(w0 + i) * 32 + lane] = (T)((word >> lane) & 1u);
            }
        } else {
            for (int i = 0; i < nw; ++i) {
                const uint32_t word = __shfl_sync(0xffffffffu, mine, i);
                row[(int64_t)(w0 + i) * 32 + lane] = (T)((word >> lane) & 1u);
            }
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

// Generations per super-step of the persistent kernel (ghost depth).  Tuning overrides, read per call:
// STC_LIFE_K = depth (1..32), STC_LIFE_COOP = 0 keeps the multi-launch kernel.
// Ghost depth of the persistent kernel (generations per neighbour exchange; STC_LIFE_K overrides):
// 8 when every SM still gets a band of at least 8 rows (4096^2: 0.97 ms per 1000 generations against
// 1.00 ms at depth 4 and 1.03 ms at 12), else 4.
static int life_coop_depth(int64_t n1, int num_sms) {
    const char* e = getenv("STC_LIFE_K");
    const int v = e ? atoi(e) : 0;
    if (v >= 1 && v <= 32) return v;
    return n1 >= 8 * (int64_t)num_sms ? 8 : 4;
}
static bool life_coop_enabled() {
    const char* e = getenv("STC_LIFE_COOP");
    return !(e && e[0] == '0');
}

template <bool C, bool WR, int WT>
static cudaError_t coop_fits_t(int grid, size_t smem, int num_sms, bool* fits) {
    auto fn = life_coop_kernel<C, WR, WT>;
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, life_threads(), smem);
    *fits = e == cudaSuccess && (int64_t)nb * num_sms >= grid;
    return e;
}

template <bool C, bool WR, int WT>
static cudaError_t coop_launch_t(const LifeCoopParams& cp, int grid, size_t smem, cudaStream_t s) {
    LifeCoopParams arg = cp;
    void* args[] = {&arg};
    return cudaLaunchCooperativeKernel((const void*)life_coop_kernel<C, WR, WT>, dim3(grid), dim3(life_threads()), args,
                                       smem, s);
}

// (fits = true: occupancy query; false: launch) for the instantiation matching (conway, wrap, W)
template <int WT>
static cudaError_t coop_dispatch_w(bool query, bool conway, bool wrap, const LifeCoopParams& cp, int grid, size_t smem,
                                   cudaStream_t s, int num_sms, bool* fits) {
    if (conway && wrap) return query ? coop_fits_t<true, true, WT>(grid, smem, num_sms, fits) : coop_launch_t<true, true, WT>(cp, grid, smem, s);
    if (conway) return query ? coop_fits_t<true, false, WT>(grid, smem, num_sms, fits) : coop_launch_t<true, false, WT>(cp, grid, smem, s);
    if (wrap) return query ? coop_fits_t<false, true, WT>(grid, smem, num_sms, fits) : coop_launch_t<false, true, WT>(cp, grid, smem, s);
    return query ? coop_fits_t<false, false, WT>(grid, smem, num_sms, fits) : coop_launch_t<false, false, WT>(cp, grid, smem, s);
}

static cudaError_t coop_dispatch(bool query, bool conway, bool wrap, const LifeCoopParams& cp, int grid, size_t smem,
                                 cudaStream_t s, int num_sms, bool* fits) {
    return cp.W == kLifeWT ? coop_dispatch_w<kLifeWT>(query, conway, wrap, cp, grid, smem, s, num_sms, fits)
                           : coop_dispatch_w<0>(query, conway, wrap, cp, grid, smem, s, num_sms, fits);
}

// The persistent path: every generation in one cooperative launch.  Returns STC_OK with *done = nsteps
// when it ran, STC_OK with *done = 0 when the grid does not suit it (caller falls back).
static int life_coop_steps(const stc_grid* a, const stc_grid* b, const stc_op* op, bool halo, bool wrap, int64_t n0,
                           int64_t n1, int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx,
                           int64_t* done) {
    *done = 0;
    if (!life_coop_enabled()) return STC_OK;
    int coop = 0;
    if (cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) != cudaSuccess || !coop) {
        cudaGetLastError();
        return STC_OK;
    }
    const int W = (int)(n0 / 32);
    int k = (int)std::min<int64_t>(life_coop_depth(n1, ctx->num_sms), std::max<int64_t>(1, nsteps - 1));
    int G = (int)std::min<int64_t>(ctx->num_sms, n1 / k);
    if (G < 1) {
        G = 1;
        k = (int)n1;
    }
    const int TBmax = (int)((n1 + G - 1) / G);
    const size_t smem = (size_t)2 * (TBmax + 2 * k) * W * 4;
    if ((int64_t)smem > ctx->max_smem_optin - 1024) return STC_OK;

    const bool conway = op->birth_mask == (1u << 3) && op->survive_mask == ((1u << 2) | (1u << 3));
    bool fits = false;
    LifeCoopParams q{};
    q.W = W;
    cudaError_t e = coop_dispatch(true, conway, wrap, q, G, smem, stream, ctx->num_sms, &fits);
    if (e != cudaSuccess) return cuda_fail(e);
    if (!fits) return STC_OK;   // not enough co-resident CTAs: the caller uses the multi-launch kernel

    const size_t words = (size_t)W * n1;
    const size_t xwords = (size_t)2 * G * 2 * k * W;
    char* mem = nullptr;
    const size_t bytes = xwords * sizeof(uint64_t) + 2 * words * sizeof(uint32_t);
    e = cudaMallocAsync((void**)&mem, bytes, stream);
    if (e != cudaSuccess) return cuda_fail(e);
    uint64_t* X = (uint64_t*)mem;
    uint32_t* P0 = (uint32_t*)(X + xwords);
    uint32_t* P1 = P0 + words;
    const int64_t org_a = halo ? 1 + a->stride[1] : 0, org_b = halo ? 1 + b->stride[1] : 0;
    int rc = launch_pack(true, a, org_a, W, (int)n1, P0, stream, ctx->num_sms);
    if (!rc) rc = cuda_fail(cudaMemsetAsync(X, 0, xwords * sizeof(uint64_t), stream));   // no stale tags
    if (rc) { cudaFreeAsync(mem, stream); return rc; }
    LifeCoopParams cp{};
    cp.in = P0;
    cp.prev = P0;
    cp.last = P1;
    cp.xbuf = X;
    cp.status = ctx->status;
    cp.W = W;
    cp.n1 = (int)n1;
    cp.k = k;
    cp.nsteps = nsteps;
    cp.birth = op->birth_mask;
    cp.survive = op->survive_mask;
    void* prof = prof_begin(stream);
    e = coop_dispatch(false, conway, wrap, cp, G, smem, stream, ctx->num_sms, &fits);
    if (e != cudaSuccess) {
        prof_end(prof, stream, "life_coop", 0.0, 0.0);
        cudaFreeAsync(mem, stream);
        return cuda_fail(e);
    }
    prof_end(prof, stream, "life_coop", 2.0 * n0 * n1 * nsteps, (double)n0 * n1 * nsteps);
    // P1 holds generation nsteps, P0 generation nsteps-1 (the input when nsteps == 1).  The reference
    // leaves the result in b after an odd number of steps, in a after an even number.
    const bool res_in_b = (nsteps & 1) != 0;
    const stc_grid* res = res_in_b ? b : a;
    const stc_grid* prev = res_in_b ? a : b;
    rc = launch_pack(false, res, res_in_b ? org_b : org_a, W, (int)n1, P1, stream, ctx->num_sms);
    if (!rc && nsteps > 1) rc = launch_pack(false, prev, res_in_b ? org_a : org_b, W, (int)n1, P0, stream, ctx->num_sms);
    cudaFreeAsync(mem, stream);
    if (rc) return rc;
    *src_is_b = res_in_b ? 1 : 0;
    *done = nsteps;
    return STC_OK;
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
    int rc = life_coop_steps(a, b, op, halo, wrap, n0, n1, nsteps, src_is_b, stream, ctx, done);
    if (rc || *done) return rc;
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
    rc = launch_pack(true, a, org_a, W, (int)n1, Pbuf[0], stream, ctx->num_sms);
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
constexpr int kNoAllocMaxWords = 512;                        // widest row: 512 words = 16384 cells

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
    if (nsteps > 0 && grids_overlap(a, b)) return STC_ERR_INVALID;
    if (op->code != STC_OP_LIFE || a->ndims != 2 || !is_moore1_2d(st)) return STC_ERR_UNSUPPORTED;
    if (!(a->dtype == STC_U8 || a->dtype == STC_BOOL || a->dtype == STC_I32 || a->dtype == STC_I64))
        return STC_ERR_UNSUPPORTED;
    const bool halo = bc->padding != STC_CONDITIONAL;
    const bool wrap = bc->boundary == STC_WRAP;
    const bool remove0 = bc->boundary == STC_REMOVE && bc->padval_int == 0;
    if (!wrap && !remove0) return STC_ERR_UNSUPPORTED;
    const int64_t n0 = a->size[0] - (halo ? 2 : 0), n1 = a->size[1] - (halo ? 2 : 0);
    if (n0 < 32 || n0 % 32 != 0 || n1 < 1) return STC_ERR_UNSUPPORTED;
    // life_block_kernel gives each thread at most one packed column once rows are 64 words or wider, so
    // rows wider than the CTA (kNoAllocMaxWords words) would leave columns uncomputed
    if (n0 / 32 > kNoAllocMaxWords || n0 / 32 > life_threads()) return STC_ERR_UNSUPPORTED;
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
