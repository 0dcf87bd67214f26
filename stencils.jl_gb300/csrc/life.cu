// life.cu — K3: bit-packed, temporally blocked outer-totalistic Moore(1) cellular automata.
//
// Replaces the loop  A = mapstencil!(rule, A::SwitchingStencilArray)  (src/gatherstencil.jl:77-83,
// src/array.jl:610-611) for 2D Moore(1) rules on UInt8 / Bool / Int32 / Int64 grids.
//
// Packed layout (column-interleaved): a row of n0 = 32 W cells becomes W 32-bit words, and bit j of
// word w is cell x = j W + w.  The left and right neighbours of every cell of word w are then the same
// bit of words w-1 and w+1 — no shifts — except across the row's two ends: the left neighbour word of
// word 0 is word W-1 rotated left by one bit (cell jW - 1 is bit j-1 of word W-1; cell -1 is cell
// n0-1 under Wrap), and the right neighbour word of word W-1 is word 0 rotated right by one.  Under
// Remove(0) the rotations become shifts that bring in a dead cell.  Two ways to split a band among
// threads: one packed column per thread (any width), with each row kept in shared memory between its two
// derived words, [left ghost | words 0 .. W-1 | right ghost] (pitch W + 2), written by the two threads
// that produce words W-1 and 0, so every thread reads its three neighbour words at fixed offsets; or,
// for rows of 128 words, one warp per row strip with four consecutive words per lane, rows stored bare,
// the words beyond a lane's run arriving by shuffle and the row ends' ghosts made on the sending lane.
//
// A launch advances every row band by up to k generations: each CTA holds full rows for its band plus
// k halo rows above and below (y-wrap, zero rows, or the neighbouring bands' rows), steps them k times
// in a shared ping-pong pair — the valid band shrinks by one row per generation — and writes the band
// back.  The 3x3 total t of every cell (2 bit planes per 3-cell sum, added by a carry-save adder) is
// formed bitwise: the column split sums each row's three words once as the row enters a rolling
// three-row window and then adds three rows; the warp-row split sums each word's three rows first and
// then adds three words.  The rule is evaluated bitwise on t (neighbours = t - centre).  The neighbour
// count is the count of nonzero neighbours, exactly what the LIFE op counts, so the result is
// bit-identical to the per-cell gather for any input values.
#include <algorithm>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "common.cuh"
#include "life.h"
#include "profile.h"

namespace stc {

constexpr int kLifeMaxThreads = 1024;

// CTA size of the Life kernels: 512 threads (16 warps; for 4096^2 the measured best of 128, 256 and 512
// with the warp-row split: 1.49, 1.10 and 0.96 ms per 1000 generations).  STC_LIFE_THREADS = 128 or 256
// overrides for the warp-row split, 1024 for the column split (a tuning knob).
static int life_threads(int W) {
    const char* e = getenv("STC_LIFE_THREADS");
    const int v = e ? atoi(e) : 0;
    if (W == 128) return (v == 128 || v == 256) ? v : 512;
    return v == 1024 ? 1024 : 512;
}

// Two ways to split a band row among threads.  WPL = 0: one packed column per thread; rows are stored
// with their two ghost words (pitch W + 2).  WPL > 0 (W = 32 WPL): one warp per row, WPL consecutive
// words per lane; the words beyond a lane's run come from the neighbouring lanes by shuffle (lanes 0 and
// 31 wrap around and rotate), so rows are stored bare (pitch W).
template <int WPL>
__host__ __device__ __forceinline__ int life_pitch(int W) { return WPL > 0 ? W : W + 2; }

__device__ __forceinline__ void full_add(uint32_t a, uint32_t b, uint32_t c, uint32_t& s, uint32_t& cy) {
    const uint32_t t = a ^ b;
    s = t ^ c;
    cy = (a & b) | (t & c);
}

// the left neighbour word of word 0 from word W-1, and the right neighbour word of word W-1 from word 0
template <bool WRAP>
__device__ __forceinline__ uint32_t ghost_left(uint32_t last) {
    return WRAP ? __funnelshift_l(last, last, 1) : last << 1;
}
template <bool WRAP>
__device__ __forceinline__ uint32_t ghost_right(uint32_t first) {
    return WRAP ? __funnelshift_r(first, first, 1) : first >> 1;
}

// word w of band row r (pitch P), with the ghost word it determines when rows carry them
template <int WPL>
__device__ __forceinline__ uint32_t& band_word(uint32_t* buf, int P, int r, int w) {
    return buf[(size_t)r * P + (WPL > 0 ? 0 : 1) + w];
}
template <bool WRAP, int WPL>
__device__ __forceinline__ void put_word(uint32_t* buf, int P, int W, int r, int w, uint32_t v) {
    band_word<WPL>(buf, P, r, w) = v;
    if (WPL == 0) {
        uint32_t* row = buf + (size_t)r * P;
        if (w == W - 1) row[0] = ghost_left<WRAP>(v);
        if (w == 0) row[W + 1] = ghost_right<WRAP>(v);
    }
}

// One source row seen from one column word: its 3-cell sums around every bit (a3 + 2 b3 = L + C + R)
// and the centre word.
struct RowV { uint32_t a3, b3, c; };

__device__ __forceinline__ RowV row_v(uint32_t l, uint32_t c, uint32_t r) {
    RowV v;
    v.a3 = l ^ c ^ r;
    v.b3 = (l & c) | (r & (l ^ c));
    v.c = c;
    return v;
}

// next state of the middle row m from the 3x3 total t = sum3(u) + sum3(m) + sum3(d), 0..9: a dead
// cell is born when its neighbour count t is in `birth`, a live one survives when t - 1 is in `survive`
template <bool CONWAY>
__device__ __forceinline__ uint32_t next_state(const RowV& u, const RowV& m, const RowV& d, uint32_t birth,
                                               uint32_t survive) {
    uint32_t t0, k0, x1, k1;
    full_add(u.a3, m.a3, d.a3, t0, k0);   // weight 1 and its carry (weight 2)
    full_add(u.b3, m.b3, d.b3, x1, k1);   // weight 2 and its carry (weight 4)
    const uint32_t t1 = x1 ^ k0;
    if constexpr (CONWAY) {
        // B3/S23: alive next iff t == 3, or t == 4 and alive.  Only t's low three bits are formed:
        // t in {3, 4} is exactly (t0^t2) & (t1^t2) (8 and 9 fail it), and t2 tells the two apart.
        const uint32_t t2 = k1 ^ (x1 & k0);
        return ((t0 ^ t2) & (t1 ^ t2)) & (~t2 | m.c);
    } else {
        const uint32_t c2 = x1 & k0;
        const uint32_t t2 = k1 ^ c2, t3 = k1 & c2;
        uint32_t out = 0;
#pragma unroll
        for (int v = 0; v <= 9; ++v) {
            const bool b = v <= 8 && ((birth >> v) & 1u);
            const bool s = v >= 1 && ((survive >> (v - 1)) & 1u);
            if (!b && !s) continue;
            const uint32_t eq = ((v & 1) ? t0 : ~t0) & ((v & 2) ? t1 : ~t1) & ((v & 4) ? t2 : ~t2) &
                                ((v & 8) ? t3 : ~t3);
            out |= eq & (b ? (s ? ~0u : ~m.c) : m.c);
        }
        return out;
    }
}

// A thread's fixed share of a band: packed column w of row strip s (of `strips`).  Columns run
// W-1, 0, 1, .., W-2 across the threads of a strip, so the two threads that write the row's ghost
// words (w == W-1 and w == 0) sit in the strip's first warp; only warps holding one of them take the
// ghost-writing variant of the row loop.
struct LifeLane {
    bool active;
    bool edge_warp;
    bool gl, gr;   // writes the left ghost (w == W-1) / the right ghost (w == 0)
    bool rl, rr;   // ragged rows: replaces the left neighbour of cell 0 / the right neighbour of cell n0-1
    int w;
    int w1, j1;    // ragged rows: cell n0-1 is bit j1 of word w1
    int s, strips;
    float inv_strips;
};

// Rows of n0 cells with 32 W > n0 (column-interleaved, so cells n0 .. 32W-1 are spare bits): W is
// chosen so at least two bits are spare, and the two layout neighbours that fall on spare bits are
// replaced when read: the right neighbour of cell n0-1 (bit j1 of its right word) by cell 0, and the
// left neighbour of cell 0 (bit 0 of its left word) by cell n0-1 — under Remove(0) by a dead cell.
__host__ __device__ __forceinline__ int life_words(int64_t n0) { return n0 % 32 == 0 ? (int)(n0 / 32) : (int)((n0 + 2 + 31) / 32); }

template <int WPL>
__device__ __forceinline__ LifeLane life_lane(int W, int n0) {
    LifeLane L;
    if constexpr (WPL > 0) {
        // one row strip per warp
        L.strips = (int)blockDim.x >> 5;
        L.inv_strips = 1.0f / (float)L.strips;
        L.s = threadIdx.x >> 5;
        L.active = true;
        L.edge_warp = false;
        L.gl = L.gr = L.rl = L.rr = false;
        L.w = L.w1 = L.j1 = 0;
        return L;
    }
    L.strips = max(1, (int)blockDim.x / W);
    L.inv_strips = 1.0f / (float)L.strips;
    const int item = threadIdx.x;
    const int c = item % W;
    L.s = item / W;
    L.active = item < W * L.strips;
    L.w = c == 0 ? W - 1 : c - 1;
    L.gl = L.active && L.w == W - 1;
    L.gr = L.active && L.w == 0;
    const bool ragged = n0 != 32 * W;
    L.w1 = (n0 - 1) % W;
    L.j1 = (n0 - 1) / W;
    L.rl = ragged && L.gr;
    L.rr = ragged && L.active && L.w == L.w1;
    L.edge_warp = __any_sync(0xffffffffu, L.gl || L.gr || L.rr);
    return L;
}

// Rows [ra, rb) of one strip: source rows ra-1 .. rb, each read as its (left, centre, right) words at
// fixed offsets and reduced to its 3-cell sums once as it enters a three-row window; the row walk is
// unrolled by three with the window's roles rotating, so nothing is copied between registers.
template <bool CONWAY, bool WRAP, int WT, bool EDGE>
__device__ __forceinline__ void life_strip(const LifeLane& L, const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int Wrt, int ra,
                                           int rb, uint32_t birth, uint32_t survive) {
    const int W = WT > 0 ? WT : Wrt;
    const int P = life_pitch<0>(W);
    const uint32_t* ps = src + (ra - 1) * P + L.w;   // left word of row ra-1; centre at +1, right at +2
    uint32_t* pd = dst + ra * P + 1 + L.w;
    auto load = [&](int q) -> RowV {
        uint32_t l = ps[q * P], c = ps[q * P + 1], r = ps[q * P + 2];
        if (EDGE) {
            const uint32_t* row = ps + q * P - L.w + 1;   // word 0 of this row
            if (L.rr) r = (r & ~(1u << L.j1)) | (WRAP ? (row[0] & 1u) << L.j1 : 0u);
            if (L.rl) l = (l & ~1u) | (WRAP ? (row[L.w1] >> L.j1) & 1u : 0u);
        }
        return row_v(l, c, r);
    };
    auto emit = [&](int q, const RowV& u, const RowV& m, const RowV& d) {
        const uint32_t nx = next_state<CONWAY>(u, m, d, birth, survive);
        pd[q * P] = nx;
        if (EDGE) {
            if (L.gl) pd[q * P - W] = ghost_left<WRAP>(nx);
            if (L.gr) pd[q * P + W] = ghost_right<WRAP>(nx);
        }
    };
    RowV v0 = load(0), v1 = load(1), v2;
    int r = ra;
    // invariant: v0 = row r-1, v1 = row r; ps at row r-1, pd at row r
    for (; r + 3 <= rb; r += 3) {
        v2 = load(2);
        emit(0, v0, v1, v2);
        v0 = load(3);
        emit(1, v1, v2, v0);
        v1 = load(4);
        emit(2, v2, v0, v1);
        ps += 3 * P;
        pd += 3 * P;
    }
    if (r < rb) {
        v2 = load(2);
        emit(0, v0, v1, v2);
        if (r + 1 < rb) {
            v0 = load(3);
            emit(1, v1, v2, v0);
        }
    }
}

template <int WPL>
__device__ __forceinline__ void ld_words(const uint32_t* p, uint32_t (&c)[WPL]) {
    if constexpr (WPL == 4) {
        const uint4 v = *(const uint4*)p;
        c[0] = v.x; c[1] = v.y; c[2] = v.z; c[3] = v.w;
    } else if constexpr (WPL == 2) {
        const uint2 v = *(const uint2*)p;
        c[0] = v.x; c[1] = v.y;
    } else {
#pragma unroll
        for (int i = 0; i < WPL; ++i) c[i] = p[i];
    }
}
template <int WPL>
__device__ __forceinline__ void st_words(uint32_t* p, const uint32_t (&c)[WPL]) {
    if constexpr (WPL == 4) *(uint4*)p = make_uint4(c[0], c[1], c[2], c[3]);
    else if constexpr (WPL == 2) *(uint2*)p = make_uint2(c[0], c[1]);
    else {
#pragma unroll
        for (int i = 0; i < WPL; ++i) p[i] = c[i];
    }
}

// Rows [ra, rb) of a band with W = 32 WPL words per row, computed by one warp: lane l holds words
// l WPL .. l WPL + WPL - 1 of every row it reads.  Each source row is read once (one vector load per
// lane) into a rolling three-row window of raw words.  Per output row the three rows are summed first,
// word by word (va + 2 vb = up + middle + down, two LOP3 per word); the 3x3 total of a word is then the
// sum of its own and its two neighbour words' column sums, the words beyond the lane's run arriving by
// shuffle (row ends: the sending lane shifts its sums by 0 or 1 bit, which is the ghost word's rotation
// or shift applied to the sums).  So a row costs its load once, not the three horizontal sums of every
// row a strip reads.
template <bool CONWAY, bool WRAP, int WPL>
__device__ __forceinline__ void life_warp_rows(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, int ra,
                                               int rb, uint32_t birth, uint32_t survive) {
    constexpr int W = 32 * WPL;
    const int lane = threadIdx.x & 31;
    const int lane_l = (lane + 31) & 31, lane_r = (lane + 1) & 31;
    // lane 31 sends word W-1's sums to lane 0 as its ghost (rotated or shifted left by one), lane 0 sends
    // word 0's to lane 31 rotated or shifted right: a shift by 0 or 1 per lane
    const uint32_t s_last = lane == 31 ? 1u : 0u, s_first = lane == 0 ? 1u : 0u;
    auto to_r = [&](uint32_t x) { return WRAP ? __funnelshift_l(x, x, s_last) : x << s_last; };
    auto to_l = [&](uint32_t x) { return WRAP ? __funnelshift_r(x, x, s_first) : x >> s_first; };
    const uint32_t* ps = src + (ra - 1) * W + lane * WPL;   // row ra-1
    uint32_t* pd = dst + ra * W + lane * WPL;
    struct RowW { uint32_t c[WPL]; };
    auto load = [&](int q) -> RowW {
        RowW r;
        ld_words<WPL>(ps + q * W, r.c);
        return r;
    };
    auto emit = [&](int q, const RowW& u, const RowW& m, const RowW& d) {
        uint32_t va[WPL], vb[WPL];
#pragma unroll
        for (int i = 0; i < WPL; ++i) {
            va[i] = u.c[i] ^ m.c[i] ^ d.c[i];
            vb[i] = (u.c[i] & m.c[i]) | (d.c[i] & (u.c[i] ^ m.c[i]));
        }
        const uint32_t la = __shfl_sync(0xffffffffu, to_r(va[WPL - 1]), lane_l);
        const uint32_t lb = __shfl_sync(0xffffffffu, to_r(vb[WPL - 1]), lane_l);
        const uint32_t ra_ = __shfl_sync(0xffffffffu, to_l(va[0]), lane_r);
        const uint32_t rb_ = __shfl_sync(0xffffffffu, to_l(vb[0]), lane_r);
        uint32_t o[WPL];
#pragma unroll
        for (int i = 0; i < WPL; ++i) {
            // the column sums of the left word, this word and the right word, as the three "rows" of
            // next_state (its fold is symmetric in the three)
            const RowV L{i ? va[i - 1] : la, i ? vb[i - 1] : lb, 0u};
            const RowV M{va[i], vb[i], m.c[i]};
            const RowV R{i < WPL - 1 ? va[i + 1] : ra_, i < WPL - 1 ? vb[i + 1] : rb_, 0u};
            o[i] = next_state<CONWAY>(L, M, R, birth, survive);
        }
        st_words<WPL>(pd + q * W, o);
    };
    RowW v0 = load(0), v1 = load(1), v2;
    int r = ra;
    for (; r + 3 <= rb; r += 3) {
        v2 = load(2);
        emit(0, v0, v1, v2);
        v0 = load(3);
        emit(1, v1, v2, v0);
        v1 = load(4);
        emit(2, v2, v0, v1);
        ps += 3 * W;
        pd += 3 * W;
    }
    if (r < rb) {
        v2 = load(2);
        emit(0, v0, v1, v2);
        if (r + 1 < rb) {
            v0 = load(3);
            emit(1, v1, v2, v0);
        }
    }
}

// Generation g of a band computes rows [max(g+1, lo_lim), min(rows-g-1, hi_lim)) — the rows whose three
// source rows are still valid, and (Remove) only rows inside the grid; rows outside it stay zero in both
// buffers — split into the lanes' strips: this lane's strip is [*ra, *rb).
__device__ __forceinline__ void life_strip_bounds(const LifeLane& L, int g, int rows, int lo_lim, int hi_lim, int* ra,
                                                  int* rb) {
    const int lo = max(g + 1, lo_lim), hi = min(rows - g - 1, hi_lim);
    const int nr = hi - lo;
    // the same monotone expression for a strip's end and the next strip's start, so the strips tile
    // [lo, hi) exactly whatever the float rounding
    *ra = lo + (int)((float)(nr * L.s) * L.inv_strips);
    *rb = (L.s == L.strips - 1) ? hi : lo + (int)((float)(nr * (L.s + 1)) * L.inv_strips);
}

// Advance a band through generations first .. kk-1 in the shared ping-pong pair (cur, oth), pitch
// life_pitch<WPL>(W): generation g reads cur when g is even, oth when odd (so with first = 1 the caller
// has already written generation 0 into oth).  Returns the buffer holding the result.  Ends with a
// barrier when it runs a generation.  `bounds` (optional): this strip's (ra, rb) for generations
// 0 .. kk-1, computed once per run instead of every generation.
template <bool CONWAY, bool WRAP, int WT, int WPL>
__device__ __forceinline__ uint32_t* life_gens(const LifeLane& L, uint32_t* cur, uint32_t* oth, int rows, int W,
                                               int kk, int lo_lim, int hi_lim, uint32_t birth, uint32_t survive,
                                               const int2* bounds = nullptr, int* status = nullptr, int first = 0) {
    if constexpr (WPL > 0) {
        if (bounds && kk == 8) {
            // a full super-step at the default depth: the eight generations unrolled, their strip bounds
            // read together up front
            int2 b[8];
#pragma unroll
            for (int g = 0; g < 8; ++g) b[g] = bounds[g];
#pragma unroll
            for (int g = 0; g < 8; ++g) {
                if (g < first) continue;
                const int ra = b[g].x, rb = b[g].y;
                if (ra < rb && STC_IN_BOUNDS(ra - 1, rows, status) && STC_IN_BOUNDS(rb, rows, status))
                    life_warp_rows<CONWAY, WRAP, WPL>((g & 1) ? oth : cur, (g & 1) ? cur : oth, ra, rb, birth, survive);
                __syncthreads();
            }
            return cur;   // an even number of generations: the result is back in cur
        }
    }
    if (first & 1) {
        uint32_t* t = cur;
        cur = oth;
        oth = t;
    }
#pragma unroll 2
    for (int g = first; g < kk; ++g) {
        int ra, rb;
        if (bounds) {
            const int2 b = bounds[g];
            ra = b.x;
            rb = b.y;
        } else {
            life_strip_bounds(L, g, rows, lo_lim, hi_lim, &ra, &rb);
        }
        // the strip reads band rows ra-1 .. rb (debug build: tested against the band)
        if (L.active && ra < rb && STC_IN_BOUNDS(ra - 1, rows, status) && STC_IN_BOUNDS(rb, rows, status)) {
            if constexpr (WPL > 0) life_warp_rows<CONWAY, WRAP, WPL>(cur, oth, ra, rb, birth, survive);
            else if (L.edge_warp) life_strip<CONWAY, WRAP, WT, true>(L, cur, oth, W, ra, rb, birth, survive);
            else life_strip<CONWAY, WRAP, WT, false>(L, cur, oth, W, ra, rb, birth, survive);
        }
        __syncthreads();
        uint32_t* t = cur;
        cur = oth;
        oth = t;
    }
    return cur;
}

// band rows [lo_lim, hi_lim) lie inside the grid (Remove); under Wrap every row does
template <bool WRAP>
__device__ __forceinline__ void band_limits(int rows, int gy_first, int n1, int* lo_lim, int* hi_lim) {
    if (WRAP) {
        *lo_lim = 1;
        *hi_lim = rows - 1;
    } else {
        *lo_lim = max(1, -gy_first);
        *hi_lim = min(rows - 1, n1 - gy_first);
    }
}

// fill band rows [0, rows) of buf from the packed grid (row gy_first + r; wrapped, or zero outside
// it) and zero the rows of `other` that lie outside the grid
template <bool WRAP, int WPL>
__device__ __forceinline__ void load_band(const uint32_t* in, uint32_t* buf, uint32_t* other, int rows, int W,
                                          int gy_first, int n1) {
    const int P = life_pitch<WPL>(W);
    for (int i = threadIdx.x; i < rows * W; i += blockDim.x) {
        const int r = i / W, w = i - r * W;
        int gy = gy_first + r;
        uint32_t v = 0;
        if (WRAP) {
            gy %= n1;
            if (gy < 0) gy += n1;
            v = in[(size_t)gy * W + w];
        } else if (gy >= 0 && gy < n1) {
            v = in[(size_t)gy * W + w];
        }
        put_word<WRAP, WPL>(buf, P, W, r, w, v);
    }
    if (!WRAP) {
        for (int i = threadIdx.x; i < rows * P; i += blockDim.x) {
            const int gy = gy_first + i / P;
            if (gy < 0 || gy >= n1) other[i] = 0u;
        }
    }
}

struct LifeParams {
    const uint32_t* in;
    uint32_t* out;
    int* status;    // debug build: bounds tests
    int n0;         // cells per row
    int W;          // words per row
    int n1;         // rows
    int TB;         // band rows written back per CTA
    int k;          // generations this launch
    int wrap;       // 1: Wrap, 0: Remove(0)
    uint32_t birth, survive;
};

// warp-row split for the compile-time widths it suits (32, 64, 128 words), else one column per thread
template <int WT>
__host__ __device__ constexpr int life_wpl() { return (WT > 0 && WT % 32 == 0 && WT / 32 <= 4 && WT / 32 != 3) ? WT / 32 : 0; }

template <bool CONWAY, bool WRAP, int WT>
__global__ void __launch_bounds__(life_wpl<WT>() > 0 ? 512 : kLifeMaxThreads, 1) life_block_kernel(const LifeParams p) {
    extern __shared__ __align__(16) uint32_t lsm[];
    constexpr int WPL = life_wpl<WT>();
    const int W = WT > 0 ? WT : p.W, P = life_pitch<WPL>(W), k = p.k;
    const int rows = p.TB + 2 * k;
    uint32_t* buf0 = lsm;
    uint32_t* buf1 = lsm + (size_t)rows * P;
    const int y0 = blockIdx.x * p.TB;
    load_band<WRAP, WPL>(p.in, buf0, buf1, rows, W, y0 - k, p.n1);
    __syncthreads();
    int lo_lim, hi_lim;
    band_limits<WRAP>(rows, y0 - k, p.n1, &lo_lim, &hi_lim);
    const LifeLane lane = life_lane<WPL>(W, p.n0);
    uint32_t* fin = life_gens<CONWAY, WRAP, WT, WPL>(lane, buf0, buf1, rows, W, k, lo_lim, hi_lim, p.birth, p.survive,
                                                     nullptr, p.status);
    for (int i = threadIdx.x; i < p.TB * W; i += blockDim.x) {
        const int r = i / W, w = i - r * W;
        const int gy = y0 + r;
        if (gy < p.n1) p.out[(size_t)gy * W + w] = band_word<WPL>(fin, P, r + k, w);
    }
}

// ------------------------------------------------------------------ persistent (cooperative) variant
// One launch runs every generation.  CTA b keeps its band (rows [y0, y1), balanced split of n1) in
// shared memory for the whole run, with k ghost rows above and below.  A super-step advances the band
// kk <= k generations; then the CTA publishes its first and last k band rows to an exchange slot in
// global memory, each word as a 64-bit (super-step tag, word) pair written with a single relaxed
// gpu-scope store.  At the next super-step every thread issues the first reads of its share of the
// neighbours' rows, computes its strip of the next generation's rows that need no ghost row (warp-row
// split) while they are in flight, reads again until each pair carries the expected tag (bounded),
// and copies the words in as ghost rows; the rows next to the ghost rows follow.  No fence or flag
// sits on the critical path: a pair is atomic, so a matching tag means the word is the
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
    int n0, W, n1, k;   // cells per row, words per row, rows, ghost depth
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

// tag of a tagged pair
__device__ __forceinline__ uint32_t tag_of(uint64_t v) { return (uint32_t)(v >> 32); }

template <bool CONWAY, bool WRAP, int WT>
__global__ void __launch_bounds__(life_wpl<WT>() > 0 ? 512 : kLifeMaxThreads, 1) life_coop_kernel(const LifeCoopParams p) {
    extern __shared__ __align__(16) uint32_t lsm[];
    constexpr int WPL = life_wpl<WT>();
    const int W = WT > 0 ? WT : p.W, P = life_pitch<WPL>(W), k = p.k, G = gridDim.x, b = blockIdx.x;
    const int y0 = (int)(((int64_t)b * p.n1) / G), y1 = (int)(((int64_t)(b + 1) * p.n1) / G);
    const int TB = y1 - y0, rows = TB + 2 * k;
    const int TBmax = (p.n1 + G - 1) / G;
    uint32_t* const buf1 = lsm + (size_t)(TBmax + 2 * k) * P;
    uint32_t* cur = lsm;
    uint32_t* oth = buf1;
    load_band<WRAP, WPL>(p.in, cur, oth, rows, W, y0 - k, p.n1);
    __syncthreads();
    int lo_lim, hi_lim;
    band_limits<WRAP>(rows, y0 - k, p.n1, &lo_lim, &hi_lim);
    const int up = b == 0 ? G - 1 : b - 1, dn = b == G - 1 ? 0 : b + 1;
    const bool has_up = WRAP || b > 0, has_dn = WRAP || b < G - 1;
    const int slab = k * W;                            // one published row block
    const int64_t nmain = p.nsteps - 1;                // generations before the last one
    const LifeLane lane = life_lane<WPL>(W, p.n0);
    // every super-step's generation g uses the same strip bounds: computed once, [strip][g]
    __shared__ int2 s_bounds[WPL > 0 ? 1024 : 1];
    __shared__ int4 s_split[WPL > 0 ? 32 : 1];
    const bool tabled = WPL > 0 && lane.strips * k <= 1024 && lane.strips <= 32;
    if (tabled) {
        for (int i = threadIdx.x; i < lane.strips * k; i += blockDim.x) {
            LifeLane t = lane;
            t.s = i / k;
            int ra, rb;
            life_strip_bounds(t, i - t.s * k, rows, lo_lim, hi_lim, &ra, &rb);
            s_bounds[i] = make_int2(ra, rb);
        }
        // generation 1 of a super-step split around the neighbour exchange: the rows whose three source
        // rows all lie in the band (computed while the exchange's first reads are in flight), then the
        // rows next to the ghost rows, the upper ones by the first half of the strips, the lower ones by
        // the second half
        if (threadIdx.x < lane.strips) {
            const int sidx = threadIdx.x, S = lane.strips, H = S / 2;
            const int lo0 = max(1, lo_lim), hi0 = min(rows - 1, hi_lim);
            int ilo = max(k + 1, lo0), ihi = min(k + TB - 1, hi0);
            if (ihi <= ilo) ilo = ihi = lo0;   // no inner rows: every row in the lower group
            int4 v;
            v.x = ilo + (ihi - ilo) * sidx / S;
            v.y = ilo + (ihi - ilo) * (sidx + 1) / S;
            if (sidx < H) {
                v.z = lo0 + (ilo - lo0) * sidx / H;
                v.w = lo0 + (ilo - lo0) * (sidx + 1) / H;
            } else {
                v.z = ihi + (hi0 - ihi) * (sidx - H) / (S - H);
                v.w = ihi + (hi0 - ihi) * (sidx - H + 1) / (S - H);
            }
            s_split[sidx] = v;
        }
        __syncthreads();
    }
    const int2* my_bounds = tabled ? s_bounds + lane.s * k : nullptr;
    // exchange reads that fit one batch per thread can overlap generation 1's inner rows
    constexpr int kB = WPL > 0 ? 2 : 4;   // pairs per thread and direction in flight (warp-row split at depth 8: 2)
    const bool split = tabled && lane.strips >= 2 && slab <= kB * (int)blockDim.x;
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
            // kB elements per thread at a time: all their first reads are in flight together, and the
            // elements whose tag is not there yet are read again together (bounded), so a super-step's
            // exchange costs about two L2 round trips when the neighbours publish at the same time
            const uint32_t want = (uint32_t)step;
            // a missing neighbour (Remove edge) reads as a zero word that already carries the tag
            const uint64_t none = (uint64_t)want << 32;
            auto first_reads = [&](int i0, uint64_t (&vu)[kB], uint64_t (&vd)[kB]) {
#pragma unroll
                for (int j = 0; j < kB; ++j) {
                    const int i = i0 + j * (int)blockDim.x;
                    vu[j] = (has_up && i < slab) ? ld_relaxed_gpu(from_up + i) : none;
                    vd[j] = (has_dn && i < slab) ? ld_relaxed_gpu(from_dn + i) : none;
                }
            };
            auto take = [&](int i0, uint64_t (&vu)[kB], uint64_t (&vd)[kB]) {
                bool ready = true;
#pragma unroll
                for (int j = 0; j < kB; ++j) ready = ready && tag_of(vu[j]) == want && tag_of(vd[j]) == want;
                if (!ready && ok) {   // after a timeout the remaining batches are not waited for
                    const long long t0 = clock64();
                    while (!ready) {
                        if (clock64() - t0 > 4000000000ll) {
                            ok = false;
                            break;
                        }
#pragma unroll
                        for (int j = 0; j < kB; ++j) {
                            const int i = i0 + j * (int)blockDim.x;
                            if (tag_of(vu[j]) != want) vu[j] = ld_relaxed_gpu(from_up + i);
                            if (tag_of(vd[j]) != want) vd[j] = ld_relaxed_gpu(from_dn + i);
                        }
                        ready = true;
#pragma unroll
                        for (int j = 0; j < kB; ++j) ready = ready && tag_of(vu[j]) == want && tag_of(vd[j]) == want;
                    }
                }
#pragma unroll
                for (int j = 0; j < kB; ++j) {
                    const int i = i0 + j * (int)blockDim.x;
                    if (i < slab) {
                        const int r = i / W, w = i - r * W;
                        put_word<WRAP, WPL>(cur, P, W, r, w, (uint32_t)vu[j]);
                        put_word<WRAP, WPL>(cur, P, W, k + TB + r, w, (uint32_t)vd[j]);
                    }
                }
            };
            if (split) {
                uint64_t vu[kB], vd[kB];
                first_reads((int)threadIdx.x, vu, vd);
                if constexpr (WPL > 0) {
                    // generation 1's inner rows read band rows only, which the exchange does not write
                    const int4 sp = s_split[lane.s];
                    if (sp.x < sp.y && STC_IN_BOUNDS(sp.x - 1, rows, p.status) && STC_IN_BOUNDS(sp.y, rows, p.status))
                        life_warp_rows<CONWAY, WRAP, WPL>(cur, oth, sp.x, sp.y, p.birth, p.survive);
                }
                take((int)threadIdx.x, vu, vd);
            } else {
                for (int i0 = threadIdx.x; i0 < slab; i0 += kB * blockDim.x) {
                    uint64_t vu[kB], vd[kB];
                    first_reads(i0, vu, vd);
                    take(i0, vu, vd);
                }
            }
            if (!__syncthreads_and(ok)) {
                if (threadIdx.x == 0 && p.status) atomicOr(p.status, DEV_ERR_TIMEOUT);
                return;
            }
            if (final && p.nsteps > 1) {
                // generation n-1: every thread has seen both neighbours' publications (so they are past
                // their initial load), and nobody reads `in` any more
                for (int i = threadIdx.x; i < TB * W; i += blockDim.x) {
                    const int r = i / W, w = i - r * W;
                    p.prev[(size_t)y0 * W + i] = band_word<WPL>(cur, P, k + r, w);
                }
            }
        }
        int first = 0;
        if constexpr (WPL > 0) {
            if (split && step > 0) {
                // generation 1's rows next to the ghost rows, now that those are in place
                const int4 sp = s_split[lane.s];
                if (sp.z < sp.w && STC_IN_BOUNDS(sp.z - 1, rows, p.status) && STC_IN_BOUNDS(sp.w, rows, p.status))
                    life_warp_rows<CONWAY, WRAP, WPL>(cur, oth, sp.z, sp.w, p.birth, p.survive);
                __syncthreads();
                first = 1;
            }
        }
        cur = life_gens<CONWAY, WRAP, WT, WPL>(lane, cur, oth, rows, W, kk, lo_lim, hi_lim, p.birth, p.survive,
                                               my_bounds, p.status, first);
        oth = (cur == lsm) ? buf1 : lsm;
        gen += kk;
        if (final) {
            for (int i = threadIdx.x; i < TB * W; i += blockDim.x) {
                const int r = i / W, w = i - r * W;
                p.last[(size_t)y0 * W + i] = band_word<WPL>(cur, P, k + r, w);
            }
            return;
        }
        uint64_t* xd = p.xbuf + (size_t)(step & 1) * G * 2 * slab + (size_t)b * 2 * slab;
        const uint64_t tag = (uint64_t)(uint32_t)(step + 1) << 32;
        for (int i = threadIdx.x; i < slab; i += blockDim.x) {
            const int r = i / W, w = i - r * W;
            st_relaxed_gpu(xd + i, tag | band_word<WPL>(cur, P, k + r, w));           // band rows y0 .. y0+k-1
            st_relaxed_gpu(xd + slab + i, tag | band_word<WPL>(cur, P, TB + r, w));   // band rows y1-k .. y1-1
        }
    }
}

// Row width specialised at compile time (128 words = 4096 cells); other widths use the run-time path.
constexpr int kLifeWT = 128;
// The warp-row split runs rows of exactly kLifeWT words with no spare bits; everything else the column split.
static bool life_split_rows(int64_t n0, int W) { return W == kLifeWT && n0 == 32ll * W; }

// A kernel's dynamic shared-memory limit only ever rises to the largest size a launch asked for, so a
// launch never finds it lowered by a smaller one (another grid, another host thread).
static cudaError_t ensure_smem_attr(const void* fn, size_t smem) {
    static std::mutex mu;
    static std::vector<std::pair<const void*, size_t>> set;
    std::lock_guard<std::mutex> g(mu);
    for (auto& f : set)
        if (f.first == fn) {
            if (f.second >= smem) return cudaSuccess;
            cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            if (e == cudaSuccess) f.second = smem;
            return e;
        }
    cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e == cudaSuccess) set.emplace_back(fn, smem);
    return e;
}

// launch one k-generation pass (both entry points use this)
template <bool C, bool WR, int WT>
static cudaError_t life_launch_t(const LifeParams& lp, int grid, size_t smem, cudaStream_t s) {
    cudaError_t e = ensure_smem_attr((const void*)life_block_kernel<C, WR, WT>, smem);
    if (e != cudaSuccess) return e;
    life_block_kernel<C, WR, WT><<<grid, life_threads(lp.W), smem, s>>>(lp);
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
    return life_split_rows(lp.n0, lp.W) ? life_launch_w<kLifeWT>(lp, conway, grid, smem, s) : life_launch_w<0>(lp, conway, grid, smem, s);
}

// bytes of shared memory for a band pair of `rows` rows of W words (the split the kernels use for W)
static size_t life_band_smem(int rows, int W, int64_t n0) {
    const int P = life_split_rows(n0, W) ? life_pitch<life_wpl<kLifeWT>()>(W) : life_pitch<0>(W);
    return (size_t)2 * rows * P * sizeof(uint32_t);
}

// ------------------------------------------------------------------ pack / unpack
struct PackParams {
    const void* base;   // parent base
    int64_t org;        // parent offset of logical (0, 0)
    int64_t sy;         // parent row stride (elements)
    int dt;
    int n0, W, n1;      // cells per row, words per row, rows
    uint32_t* P;
};

// one thread per packed word: bit j of word (y, w) is cell (j W + w, y), so the 32 reads of a warp's
// threads for one j are consecutive cells
template <class T>
__global__ void life_pack_kernel(const PackParams p) {
    const T* base = (const T*)p.base;
    const int64_t nwords = (int64_t)p.n1 * p.W;
    for (int64_t gi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; gi < nwords; gi += (int64_t)gridDim.x * blockDim.x) {
        const int y = (int)(gi / p.W), w = (int)(gi - (int64_t)y * p.W);
        const T* cell = base + p.org + (int64_t)y * p.sy + w;
        bool nz[32];
#pragma unroll
        for (int j = 0; j < 32; ++j) nz[j] = j * p.W + w < p.n0 && cell[(int64_t)j * p.W] != (T)0;   // spare bits 0
        uint32_t v = 0;
#pragma unroll
        for (int j = 0; j < 32; ++j) v |= (uint32_t)nz[j] << j;
        p.P[gi] = v;
    }
}

template <class T>
__global__ void life_unpack_kernel(const PackParams p) {
    T* base = (T*)p.base;
    const int64_t nwords = (int64_t)p.n1 * p.W;
    for (int64_t gi = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; gi < nwords; gi += (int64_t)gridDim.x * blockDim.x) {
        const int y = (int)(gi / p.W), w = (int)(gi - (int64_t)y * p.W);
        T* cell = base + p.org + (int64_t)y * p.sy + w;
        const uint32_t v = p.P[gi];
#pragma unroll
        for (int j = 0; j < 32; ++j)
            if (j * p.W + w < p.n0) cell[(int64_t)j * p.W] = (T)((v >> j) & 1u);
    }
}

// Byte grids (UInt8, Bool) whose rows are whole packed words (n0 = 32 W, W a multiple of 32) on 16-byte
// aligned rows: one warp packs 32 words of a row at a time.  Lane j reads cells j W + 32 c .. j W + 32 c + 31
// (one 32-byte sector, two 16-byte loads); byte b of lane j is bit j of word 32 c + b, so one ballot per byte
// forms a whole word, and the 32 words leave as one 128-byte store.  Unpacking is the mirror image: every
// lane reads the same 32 words and writes its 32 cells as one sector.  (The one-thread-per-word kernels
// above need 32 one-byte accesses per word.)
__global__ void life_pack_bytes_kernel(const PackParams p) {
    const uint8_t* base = (const uint8_t*)p.base;
    const int lane = threadIdx.x & 31;
    const int G = p.W / 32;
    const int64_t units = (int64_t)p.n1 * G;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < units; u += nw) {
        const int y = (int)(u / G), c = (int)(u - (int64_t)y * G);
        const uint4* src = (const uint4*)(base + p.org + (int64_t)y * p.sy + (int64_t)lane * p.W + 32 * c);
        const uint4 v0 = src[0], v1 = src[1];
        const uint32_t q[8] = {v0.x, v0.y, v0.z, v0.w, v1.x, v1.y, v1.z, v1.w};
        uint32_t mine = 0;
#pragma unroll
        for (int b = 0; b < 32; ++b) {
            const uint32_t word = __ballot_sync(0xffffffffu, ((q[b >> 2] >> (8 * (b & 3))) & 0xffu) != 0u);
            if (lane == b) mine = word;
        }
        p.P[(int64_t)y * p.W + 32 * c + lane] = mine;
    }
}

__global__ void life_unpack_bytes_kernel(const PackParams p) {
    uint8_t* base = (uint8_t*)p.base;
    const int lane = threadIdx.x & 31;
    const int G = p.W / 32;
    const int64_t units = (int64_t)p.n1 * G;
    const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
    for (int64_t u = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5; u < units; u += nw) {
        const int y = (int)(u / G), c = (int)(u - (int64_t)y * G);
        // each lane takes its bit of the 32 words: one word per lane, then shuffled round
        const uint32_t word = p.P[(int64_t)y * p.W + 32 * c + lane];
        uint32_t o[8];
#pragma unroll
        for (int i = 0; i < 8; ++i) {
            o[i] = 0;
#pragma unroll
            for (int bb = 0; bb < 4; ++bb)
                o[i] |= ((__shfl_sync(0xffffffffu, word, 4 * i + bb) >> lane) & 1u) << (8 * bb);
        }
        uint4* dst = (uint4*)(base + p.org + (int64_t)y * p.sy + (int64_t)lane * p.W + 32 * c);
        dst[0] = make_uint4(o[0], o[1], o[2], o[3]);
        dst[1] = make_uint4(o[4], o[5], o[6], o[7]);
    }
}

static int launch_pack(bool pack, const stc_grid* g, int64_t org, int64_t n0, int W, int n1, uint32_t* P,
                       cudaStream_t s, int num_sms) {
    PackParams p{};
    p.base = g->data;
    p.org = org;
    p.sy = g->stride[1];
    p.dt = g->dtype;
    p.n0 = (int)n0;
    p.W = W;
    p.n1 = n1;
    p.P = P;
    const bool bytes_fast = (g->dtype == STC_U8 || g->dtype == STC_BOOL) && n0 == 32ll * W && W % 32 == 0 &&
                            ((uintptr_t)((const uint8_t*)g->data + org) % 16) == 0 && g->stride[1] % 16 == 0;
    if (bytes_fast) {
        const int64_t warps = (int64_t)n1 * (W / 32);
        const int blocks = (int)std::max<int64_t>(1, std::min<int64_t>((warps + 7) / 8, (int64_t)num_sms * 16));
        void* prof = prof_begin(s);
        if (pack) life_pack_bytes_kernel<<<blocks, 256, 0, s>>>(p);
        else life_unpack_bytes_kernel<<<blocks, 256, 0, s>>>(p);
        prof_end(prof, s, pack ? "life_pack" : "life_unpack", (double)W * 32 * n1 * 1.125, (double)W * 32 * n1);
        return cuda_fail(cudaGetLastError());
    }
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
void life_plan(int W, int64_t n0, int n1, int64_t steps_left, int smem_cap, int num_sms, int* TB, int* k) {
    int kk = (int)std::min<int64_t>(steps_left, 16);
    int tb = std::max(8, (n1 + num_sms - 1) / num_sms);
    while (kk > 1 && (int64_t)life_band_smem(tb + 2 * kk, W, n0) > smem_cap) --kk;
    while (tb > 1 && (int64_t)life_band_smem(tb + 2 * kk, W, n0) > smem_cap) --tb;
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
static cudaError_t coop_fits_t(int W, int grid, size_t smem, int num_sms, bool* fits) {
    auto fn = life_coop_kernel<C, WR, WT>;
    cudaError_t e = ensure_smem_attr((const void*)fn, smem);
    if (e != cudaSuccess) return e;
    int nb = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, fn, life_threads(W), smem);
    *fits = e == cudaSuccess && (int64_t)nb * num_sms >= grid;
    return e;
}

template <bool C, bool WR, int WT>
static cudaError_t coop_launch_t(const LifeCoopParams& cp, int grid, size_t smem, cudaStream_t s) {
    cudaError_t e = ensure_smem_attr((const void*)life_coop_kernel<C, WR, WT>, smem);
    if (e != cudaSuccess) return e;
    LifeCoopParams arg = cp;
    void* args[] = {&arg};
    return cudaLaunchCooperativeKernel((const void*)life_coop_kernel<C, WR, WT>, dim3(grid), dim3(life_threads(cp.W)), args,
                                       smem, s);
}

// (fits = true: occupancy query; false: launch) for the instantiation matching (conway, wrap, W)
template <int WT>
static cudaError_t coop_dispatch_w(bool query, bool conway, bool wrap, const LifeCoopParams& cp, int grid, size_t smem,
                                   cudaStream_t s, int num_sms, bool* fits) {
    if (conway && wrap) return query ? coop_fits_t<true, true, WT>(cp.W, grid, smem, num_sms, fits) : coop_launch_t<true, true, WT>(cp, grid, smem, s);
    if (conway) return query ? coop_fits_t<true, false, WT>(cp.W, grid, smem, num_sms, fits) : coop_launch_t<true, false, WT>(cp, grid, smem, s);
    if (wrap) return query ? coop_fits_t<false, true, WT>(cp.W, grid, smem, num_sms, fits) : coop_launch_t<false, true, WT>(cp, grid, smem, s);
    return query ? coop_fits_t<false, false, WT>(cp.W, grid, smem, num_sms, fits) : coop_launch_t<false, false, WT>(cp, grid, smem, s);
}

static cudaError_t coop_dispatch(bool query, bool conway, bool wrap, const LifeCoopParams& cp, int grid, size_t smem,
                                 cudaStream_t s, int num_sms, bool* fits) {
    return life_split_rows(cp.n0, cp.W) ? coop_dispatch_w<kLifeWT>(query, conway, wrap, cp, grid, smem, s, num_sms, fits)
                           : coop_dispatch_w<0>(query, conway, wrap, cp, grid, smem, s, num_sms, fits);
}

// The co-residency answer (and the shared-memory attribute it sets) per (device, instantiation, grid,
// shared memory): asked once, not on every call.
static cudaError_t coop_fits_cached(bool conway, bool wrap, int n0, int W, int G, size_t smem, cudaStream_t stream,
                                    DeviceCtx* ctx, bool* fits) {
    struct Entry { int dev; bool conway, wrap, split; int G, threads; size_t smem; bool fits; };
    static std::mutex mu;
    static std::vector<Entry> cache;
    const bool split = life_split_rows(n0, W);
    const int threads = life_threads(W);
    {
        std::lock_guard<std::mutex> g(mu);
        for (const Entry& c : cache)
            if (c.dev == ctx->device && c.conway == conway && c.wrap == wrap && c.split == split && c.G == G &&
                c.threads == threads && c.smem == smem) {
                *fits = c.fits;
                return cudaSuccess;
            }
    }
    LifeCoopParams q{};
    q.n0 = n0;
    q.W = W;
    cudaError_t e = coop_dispatch(true, conway, wrap, q, G, smem, stream, ctx->num_sms, fits);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(mu);
    if (cache.size() < 256) cache.push_back(Entry{ctx->device, conway, wrap, split, G, threads, smem, *fits});
    return cudaSuccess;
}

// The persistent path: every generation in one cooperative launch.  Returns STC_OK with *done = nsteps
// when it ran, STC_OK with *done = 0 when the grid does not suit it (caller falls back).
static int life_coop_steps(const stc_grid* a, const stc_grid* b, const stc_op* op, bool halo, bool wrap, int64_t n0,
                           int64_t n1, int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx,
                           int64_t* done) {
    *done = 0;
    if (!life_coop_enabled()) return STC_OK;
    static int coop_attr[64];   // per device: 0 unknown, 1 cooperative launch supported, 2 not
    if (ctx->device >= 0 && ctx->device < 64 && coop_attr[ctx->device] == 0) {
        int coop = 0;
        const bool ok = cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device) == cudaSuccess && coop;
        cudaGetLastError();
        coop_attr[ctx->device] = ok ? 1 : 2;
    }
    if (ctx->device < 0 || ctx->device >= 64 || coop_attr[ctx->device] != 1) return STC_OK;
    const int W = life_words(n0);
    int k = (int)std::min<int64_t>(life_coop_depth(n1, ctx->num_sms), std::max<int64_t>(1, nsteps - 1));
    int G = (int)std::min<int64_t>(ctx->num_sms, n1 / k);
    if (G < 1) {
        G = 1;
        k = (int)n1;
    }
    const int TBmax = (int)((n1 + G - 1) / G);
    const size_t smem = life_band_smem(TBmax + 2 * k, W, n0);
    if ((int64_t)smem > ctx->max_smem_optin - 1024) return STC_OK;

    const bool conway = op->birth_mask == (1u << 3) && op->survive_mask == ((1u << 2) | (1u << 3));
    bool fits = false;
    cudaError_t e = coop_fits_cached(conway, wrap, (int)n0, W, G, smem, stream, ctx, &fits);
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
    int rc = launch_pack(true, a, org_a, n0, W, (int)n1, P0, stream, ctx->num_sms);
    if (!rc) rc = cuda_fail(cudaMemsetAsync(X, 0, xwords * sizeof(uint64_t), stream));   // no stale tags
    if (rc) { cudaFreeAsync(mem, stream); return rc; }
    LifeCoopParams cp{};
    cp.in = P0;
    cp.prev = P0;
    cp.last = P1;
    cp.xbuf = X;
    cp.status = status_slot(ctx, stream).dev;
    cp.n0 = (int)n0;
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
    rc = launch_pack(false, res, res_in_b ? org_b : org_a, n0, W, (int)n1, P1, stream, ctx->num_sms);
    if (!rc && nsteps > 1) rc = launch_pack(false, prev, res_in_b ? org_a : org_b, n0, W, (int)n1, P0, stream, ctx->num_sms);
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
    if (n0 < 32 || n1 < 1 || life_words(n0) > 512 || n1 > (1 << 30)) return STC_OK;
    int rc = life_coop_steps(a, b, op, halo, wrap, n0, n1, nsteps, src_is_b, stream, ctx, done);
    if (rc || *done) return rc;
    const int W = life_words(n0);
    const int smem_cap = ctx->max_smem_optin - 1024;
    int TB, k;
    life_plan(W, n0, (int)n1, nsteps, smem_cap, ctx->num_sms, &TB, &k);
    if ((int64_t)life_band_smem(TB + 2 * k, W, n0) > smem_cap) return STC_OK;

    const size_t words = (size_t)W * n1;
    uint32_t* P = nullptr;
    cudaError_t e = cudaMallocAsync((void**)&P, 2 * words * sizeof(uint32_t), stream);
    if (e != cudaSuccess) return cuda_fail(e);
    uint32_t* Pbuf[2] = {P, P + words};
    const int64_t org_a = halo ? 1 + a->stride[1] : 0, org_b = halo ? 1 + b->stride[1] : 0;
    rc = launch_pack(true, a, org_a, n0, W, (int)n1, Pbuf[0], stream, ctx->num_sms);
    if (rc) { cudaFreeAsync(P, stream); return rc; }

    LifeParams lp{};
    lp.status = status_slot(ctx, stream).dev;
    lp.n0 = (int)n0;
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
        life_plan(W, n0, (int)n1, budget, smem_cap, ctx->num_sms, &TB, &k);
        lp.in = Pbuf[cur];
        lp.out = Pbuf[1 - cur];
        lp.TB = TB;
        lp.k = k;
        const size_t smem = life_band_smem(TB + 2 * k, W, n0);
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
    rc = launch_pack(false, res, res_in_b ? org_b : org_a, n0, W, (int)n1, Pbuf[cur], stream, ctx->num_sms);
    if (!rc && nsteps > 1) rc = launch_pack(false, prev, res_in_b ? org_a : org_b, n0, W, (int)n1, Pbuf[1 - cur], stream, ctx->num_sms);
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

static int noalloc_pack_launch(bool pack, const stc_grid* g, int64_t org, int64_t n0, int W, int n1, uint32_t* P,
                               cudaStream_t s, int num_sms) {
    PackParams p{};
    p.base = g->data;
    p.org = org;
    p.sy = g->stride[1];
    p.dt = g->dtype;
    p.n0 = (int)n0;
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
    if (n0 < 32 || n1 < 1) return STC_ERR_UNSUPPORTED;
    // life_block_kernel gives each thread one packed column of a strip, so rows wider than the CTA
    // (kNoAllocMaxWords words) would leave columns uncomputed
    if (life_words(n0) > kNoAllocMaxWords || life_words(n0) > life_threads(life_words(n0))) return STC_ERR_UNSUPPORTED;
    if ((int64_t)life_words(n0) * 32 * n1 > kNoAllocMaxCells) return STC_ERR_TOO_LARGE;   // packed words fit
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
    const int W = life_words(n0);
    const int smem_cap = smem_optin - 1024;
    int TB, k;
    life_plan(W, n0, (int)n1, nsteps, smem_cap, num_sms, &TB, &k);
    if ((int64_t)life_band_smem(TB + 2 * k, W, n0) > smem_cap) return STC_ERR_UNSUPPORTED;
    uint32_t* Pbuf[2] = {P, P + kNoAllocWords};
    const int64_t org_a = halo ? 1 + a->stride[1] : 0, org_b = halo ? 1 + b->stride[1] : 0;
    if ((rc = noalloc_pack_launch(true, a, org_a, n0, W, (int)n1, Pbuf[0], s, num_sms))) return rc;
    LifeParams lp{};
    lp.n0 = (int)n0;
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
        life_plan(W, n0, (int)n1, budget, smem_cap, num_sms, &TB, &k);
        lp.in = Pbuf[cur];
        lp.out = Pbuf[1 - cur];
        lp.TB = TB;
        lp.k = k;
        const size_t smem = life_band_smem(TB + 2 * k, W, n0);
        const int grid = (int)((n1 + TB - 1) / TB);
        if ((e = life_launch(lp, conway, grid, smem, s)) != cudaSuccess) return cuda_fail(e);
        cur = 1 - cur;
        left -= k;
    }
    const bool res_in_b = (nsteps & 1) != 0;
    const stc_grid* res = res_in_b ? b : a;
    const stc_grid* prev = res_in_b ? a : b;
    if ((rc = noalloc_pack_launch(false, res, res_in_b ? org_b : org_a, n0, W, (int)n1, Pbuf[cur], s, num_sms))) return rc;
    if (nsteps > 1 &&
        (rc = noalloc_pack_launch(false, prev, res_in_b ? org_a : org_b, n0, W, (int)n1, Pbuf[1 - cur], s, num_sms)))
        return rc;
    if (out_src_is_b) *out_src_is_b = res_in_b ? 1 : 0;
    return cuda_fail(cudaStreamSynchronize(s));
}
