// tblock3d.cu — K6: temporally blocked multi-step maps on 3D grids.
//
// Replaces k iterations of  A = mapstencil!(f, A)  (src/gatherstencil.jl:77-83, switch src/array.jl:610-611)
// for 3D radius-1 stencils whose off-plane taps are the two cells straight above and below
// (VonNeumann(1,3): the 7-point diffusion; Cross(1,3)), on Float32 / BFloat16 / Float16 state.
//
// The run works on an internal pair of parents padded by a ring of H cells (H >= k, the row start of
// the interior on a 128-byte line); before every pass the ring holds the boundary's values (Wrap:
// refreshed by K2 from the interior; Remove: padval, written once), so every input box arrives whole
// from TMA and no tile needs patching.
//
// A CTA owns an (x, y) tile of TX x TY outputs plus a halo (XH columns, K rows each side: the plane
// box BX x BY) and a chunk of ZC output planes.  Input planes stream through a 5-slot TMA ring
// (cp.async.bulk.tensor.3d, one plane per copy, two planes ahead, no multicast).  At iteration i time
// level t computes its plane i - t from level t-1's planes i-t-1, i-t and i-t+1.  Every thread owns
// the same 4 x RPT block of each level's plane.  The plane at a cell's own height is read from shared
// memory (two parity buffers per level, so one barrier per iteration suffices); the plane below is the
// one the thread read there in the previous iteration (kept in registers); the plane above is the one
// the level below produced earlier in the same iteration (registers).  Left / right neighbours arrive
// by warp shuffle from the adjacent lanes.  Level 1 reads the input planes from the ring.  Level k
// writes the tile's interior to the other parent, so a pass over HBM advances the grid k steps.
//
// Cells outside the grid: with Wrap the ring is the periodic extension of the grid and evolves
// exactly like the cells it copies (same inputs, same fold), so nothing is patched; with Remove every
// level writes padval there, as getneighbor does at every step (src/array.jl:129-137).  Every cell
// update is the single-map fold (the same op structs over Float32, widened as in K1's vector path), and
// in the default mode every level is rounded to the storage type, so results are bit-identical to k
// separate maps.  With STC_KEEP_F32 (16-bit storage only) the levels inside a pass stay Float32 and
// only the states written to memory are rounded (BFloat16: stochastically, from a hash of the cell and
// the step; Float16: to nearest), on the schedule the header states.
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

constexpr int kTbK = 4;              // time levels per pass (8 for BFloat16 in the STC_KEEP_F32 mode)
constexpr int kTbKMax = 8;
constexpr int kTbRPT = 2;            // rows per thread block (the thread owns 4 x kTbRPT cells of a plane)
constexpr int kTbRing = 5;           // input planes resident: i-2 .. i (read) and i+1, i+2 (in flight)
constexpr int kTbMaxThreads = 512;   // 16 warps: four per SM sub-partition, up to 128 registers each

struct TB6Params {
    CUtensorMap tmap;                // the padded source buffer (rank 3), box BX x BY x 1
    void* dst;                       // padded destination buffer: element of logical (0, 0, 0)
    int64_t dstr1, dstr2;            // its strides (elements)
    int32_t n[3];                    // logical size
    int32_t H;                       // ring width: tensor-map coordinate of logical 0 on every axis
    int32_t BX, BY;                  // plane box
    int32_t XH;                      // box column of the tile's first column (>= K, multiple of 4)
    int32_t TX, TY, ZC;              // tile and z chunk (outputs)
    int32_t ntx, nty, nzc, nitems;
    int32_t remove;                  // Remove: cells outside the grid hold padval at every level
    float padf;                      // padval in the storage type, widened
    uint32_t box_bytes;              // BX * BY * sizeof(T): one TMA transaction
    uint32_t ring_off, ring_stride;  // byte offset of ring slot 0 and bytes per slot
    uint32_t lvl_off, lvl_stride;    // byte offset of the level buffers and bytes per buffer
    uint32_t bar_off;
    int32_t keep_f32;                // levels inside the pass stay Float32 (16-bit storage only)
    int32_t stochastic;              // round the stored level stochastically (BFloat16)
    uint32_t round_step;             // the step number the stored level reaches (hash input)
    int32_t* status;
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

// The same op over Float32 inputs and Float32 results (no rounding to the storage type).
template <class Op> struct TbF32;
template <class Tin, class Tout> struct TbF32<OpDiffuse<Tin, Tout, float>> { using type = OpDiffuse<float, float, float>; };
template <class Tin, class Tout> struct TbF32<OpMean<Tin, Tout, float>> { using type = OpMean<float, float, float>; };
template <class Tin, class Tout> struct TbF32<OpSumF<Tin, Tout, float>> { using type = OpSumF<float, float, float>; };

// Which taps the table has, as compile-time scalars: the kernel reads only those neighbours.
template <class Sh> struct TbTaps {
    static constexpr bool has(int x, int y, int z) {
        for (int k = 0; k < Sh::L; ++k)
            if (Sh::table.o[k].x == x && Sh::table.o[k].y == y && Sh::table.o[k].z == z) return true;
        return false;
    }
    static constexpr bool only_axis_taps() {
        for (int k = 0; k < Sh::L; ++k) {
            const auto o = Sh::table.o[k];
            const int nz = (o.x != 0) + (o.y != 0) + (o.z != 0);
            if (nz > 1 || o.x < -1 || o.x > 1 || o.y < -1 || o.y > 1 || o.z < -1 || o.z > 1) return false;
        }
        return true;
    }
    static constexpr bool kUp = has(0, -1, 0), kDn = has(0, 1, 0), kLf = has(-1, 0, 0), kRt = has(1, 0, 0);
};

template <class T> __device__ __forceinline__ float tb_widen(T v) {
    if constexpr (std::is_same_v<T, float>) return v;
    else if constexpr (std::is_same_v<T, __nv_bfloat16>) return __bfloat162float(v);
    else return __half2float(v);
}

// "lowbias32" integer hash (Chris Wellons, hash-prospector; public domain): the source of the rounding
// bits of the stochastic BFloat16 store.  The oracle computes the same bits.
__device__ __forceinline__ uint32_t tb_mix(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}

// Float32 -> BFloat16 with stochastic rounding: the 16 bits below the BFloat16 mantissa are added to
// the magnitude and the sum truncated, so a value rounds up with probability equal to its distance
// from the value below.  The 16 random bits come from the hash of the cell's column-major linear index
// and the step number.  Infinities and NaN round to nearest.
__device__ __forceinline__ __nv_bfloat16 tb_bf16_stochastic(float v, uint64_t lin, uint32_t step) {
    uint32_t b = __float_as_uint(v);
    if ((b & 0x7f800000u) == 0x7f800000u) return __float2bfloat16_rn(v);
    const uint32_t h = tb_mix((uint32_t)lin ^ tb_mix((uint32_t)(lin >> 32) ^ tb_mix(step ^ 0x9e3779b9u)));
    b += h & 0xffffu;
    return __ushort_as_bfloat16((unsigned short)(b >> 16));
}

template <class T> __device__ __forceinline__ T tb_round(float v);
template <> __device__ __forceinline__ float tb_round<float>(float v) { return v; }
template <> __device__ __forceinline__ __nv_bfloat16 tb_round<__nv_bfloat16>(float v) { return __float2bfloat16_rn(v); }
template <> __device__ __forceinline__ __half tb_round<__half>(float v) { return __float2half_rn(v); }

// four consecutive storage elements (an aligned 4 * sizeof(T)-byte group) to global memory
template <class T> __device__ __forceinline__ void tb_st4(T* d, const T* v) {
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

// One level's RPT x 4 cells.  M: the cells at their own height (level t-1), LO / HI: the cells below /
// above; UP / DN: the row above / below the block, LF / RT: the column left / right of it (all level
// t-1, plane p).  Every cell folds its taps in table order.
template <class OpF, class Sh, class P>
__device__ __forceinline__ void tb_fold_block(const float (&M)[kTbRPT][4], const float (&LO)[kTbRPT][4],
                                              const float (&HI)[kTbRPT][4], const float (&UP)[4], const float (&DN)[4],
                                              const float (&LF)[kTbRPT], const float (&RT)[kTbRPT], const P& p,
                                              float (&res)[kTbRPT][4]) {
    constexpr auto Tb = Sh::table;
#pragma unroll
    for (int r = 0; r < kTbRPT; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            typename OpF::A acc;
            if constexpr (OpF::kZeroInit) acc = OpF::first(0.0f, 0);
#pragma unroll
            for (int k = 0; k < Sh::L; ++k) {
                const int dx = Tb.o[k].x, dy = Tb.o[k].y, dz = Tb.o[k].z;
                float v;
                if (dz < 0) v = LO[r][c];
                else if (dz > 0) v = HI[r][c];
                else if (dy < 0) v = r == 0 ? UP[c] : M[r - 1][c];
                else if (dy > 0) v = r == kTbRPT - 1 ? DN[c] : M[r + 1][c];
                else if (dx < 0) v = c == 0 ? LF[r] : M[r][c - 1];
                else if (dx > 0) v = c == 3 ? RT[r] : M[r][c + 1];
                else v = M[r][c];
                if (!OpF::kZeroInit && k == 0) acc = OpF::first(v, 0);
                else acc = OpF::step(acc, v, k, p);
            }
            res[r][c] = OpF::finish(acc, M[r][c], p);
        }
}

// Packed Float32 add (two lanes per instruction, add.rn.f32x2): each lane rounds exactly as __fadd_rn.
// Only the tap sums use it.  A packed multiply followed by a packed add was measured to come out fused
// (one rounding) even with an explicit rounding modifier and -fmad=false, so the finishing arithmetic
// (which multiplies) stays on the scalar __fmul_rn / __fadd_rn intrinsics, which are never fused.
__device__ __forceinline__ float2 tb_add2(float2 a, float2 b) {
    float2 r;
    asm("{\n\t.reg .b64 ra, rb, rd;\n\t"
        "mov.b64 ra, {%2, %3};\n\t"
        "mov.b64 rb, {%4, %5};\n\t"
        "add.rn.f32x2 rd, ra, rb;\n\t"
        "mov.b64 {%0, %1}, rd;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
    return r;
}

// Ops whose fold is a left fold of adds from the first tap (sum, mean, diffusion): their tap sums can
// run two cells at a time.  Pairs are the cells (0, 1) and (2, 3) of a row.
template <class OpF> struct TbPairOp { static constexpr bool kPair = false; };
template <> struct TbPairOp<OpDiffuse<float, float, float>> { static constexpr bool kPair = true; };
template <> struct TbPairOp<OpSumF<float, float, float>> { static constexpr bool kPair = true; };
template <> struct TbPairOp<OpMean<float, float, float>> { static constexpr bool kPair = true; };

template <class OpF, class Sh, class P>
__device__ __forceinline__ void tb_fold_block2(const float (&M)[kTbRPT][4], const float (&LO)[kTbRPT][4],
                                               const float (&HI)[kTbRPT][4], const float (&UP)[4], const float (&DN)[4],
                                               const float (&LF)[kTbRPT], const float (&RT)[kTbRPT], const P& p,
                                               float (&res)[kTbRPT][4]) {
    constexpr auto Tb = Sh::table;
#pragma unroll
    for (int r = 0; r < kTbRPT; ++r)
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int c = 2 * h;
            float2 acc = make_float2(0.0f, 0.0f);
#pragma unroll
            for (int k = 0; k < Sh::L; ++k) {
                const int dx = Tb.o[k].x, dy = Tb.o[k].y, dz = Tb.o[k].z;
                float2 v;
                if (dz < 0) v = make_float2(LO[r][c], LO[r][c + 1]);
                else if (dz > 0) v = make_float2(HI[r][c], HI[r][c + 1]);
                else if (dy < 0) v = r == 0 ? make_float2(UP[c], UP[c + 1]) : make_float2(M[r - 1][c], M[r - 1][c + 1]);
                else if (dy > 0) v = r == kTbRPT - 1 ? make_float2(DN[c], DN[c + 1]) : make_float2(M[r + 1][c], M[r + 1][c + 1]);
                else if (dx < 0) v = make_float2(c == 0 ? LF[r] : M[r][c - 1], M[r][c]);
                else if (dx > 0) v = make_float2(M[r][c + 1], c == 2 ? RT[r] : M[r][c + 2]);
                else v = make_float2(M[r][c], M[r][c + 1]);
                acc = k == 0 ? v : tb_add2(acc, v);
            }
            res[r][c] = OpF::finish(acc.x, M[r][c], p);
            res[r][c + 1] = OpF::finish(acc.y, M[r][c + 1], p);
        }
}

// The block's rows above / below on plane `pl` (row pitch BX elements of type S), and the one column
// each end lane of a warp needs beyond its block (edge_off: lane 31 reads right of its block, every
// other lane left of lane 0's block, so the load is a broadcast).  Rows above / below the plane and the
// columns beyond its ends read slack memory: those cells lie outside every level's valid region.
template <class S, class Sh>
__device__ __forceinline__ void tb_edges(const S* pl, int BX, int cx, int cy, int edge_off, float (&UP)[4],
                                         float (&DN)[4], float (&EDGE)[kTbRPT]) {
    using U = TbTaps<Sh>;
    if constexpr (U::kUp) ld_row_vec<S, float, 4>(pl + (cy - 1) * BX + cx, UP);
    if constexpr (U::kDn) ld_row_vec<S, float, 4>(pl + (cy + kTbRPT) * BX + cx, DN);
    if constexpr (U::kLf || U::kRt) {
#pragma unroll
        for (int r = 0; r < kTbRPT; ++r) EDGE[r] = tb_widen<S>(pl[edge_off + r * BX]);
    }
}

template <class S>
__device__ __forceinline__ void tb_own(const S* pl, int BX, int cx, int cy, float (&V)[kTbRPT][4]) {
#pragma unroll
    for (int r = 0; r < kTbRPT; ++r) ld_row_vec<S, float, 4>(pl + (cy + r) * BX + cx, V[r]);
}

// left / right columns of the block from the neighbouring lanes' cells (lanes hold consecutive blocks of
// a row band), the warp's end lanes from EDGE
template <class Sh>
__device__ __forceinline__ void tb_sides(const float (&M)[kTbRPT][4], const float (&EDGE)[kTbRPT], int lane,
                                         float (&LF)[kTbRPT], float (&RT)[kTbRPT]) {
    using U = TbTaps<Sh>;
#pragma unroll
    for (int r = 0; r < kTbRPT; ++r) {
        if constexpr (U::kLf) {
            const float v = __shfl_up_sync(0xffffffffu, M[r][3], 1);
            LF[r] = lane == 0 ? EDGE[r] : v;
        }
        if constexpr (U::kRt) {
            const float v = __shfl_down_sync(0xffffffffu, M[r][0], 1);
            RT[r] = lane == 31 ? EDGE[r] : v;
        }
    }
}

template <class T, class Op, class Sh, int K>
__global__ void __launch_bounds__(kTbMaxThreads, 1) tb6_kernel(const __grid_constant__ TB6Params p) {
    static_assert(TbTaps<Sh>::only_axis_taps(), "taps must be the centre or one step along one axis");
    using OpF = typename TbF32<Op>::type;
    extern __shared__ __align__(128) unsigned char tsm[];
    const int BX = p.BX, QX = BX >> 2;
    constexpr int k = K;
    auto ring = [&](uint32_t g) { return (const T*)(tsm + p.ring_off + (size_t)(g % kTbRing) * p.ring_stride); };
    // level buffer (t, parity): plane pointer (one slack row precedes it)
    auto lvl = [&](int t, int par) {
        return (float*)(tsm + p.lvl_off + (size_t)(2 * (t - 1) + par) * p.lvl_stride) + BX;
    };
    uint64_t* bars = (uint64_t*)(tsm + p.bar_off);

    // Threads past the last block compute a copy of a real block (so that every lane of a warp takes
    // part in the shuffles) and store nothing.
    const int nqy = p.BY / kTbRPT;
    const int nblk = QX * nqy;
    const int tid = threadIdx.x, lane = tid & 31;
    const bool act = tid < nblk;
    const int qx = tid % QX, qy = min(tid / QX, nqy - 1);
    const int cx = 4 * qx, cy = kTbRPT * qy;
    const int t0 = tid & ~31;
    const int cx0 = 4 * (t0 % QX), cy0 = kTbRPT * min(t0 / QX, nqy - 1);
    const int edge_off = lane == 31 ? cy * BX + cx + 4 : cy0 * BX + cx0 - 1;

    if (tid == 0) {
        prefetch_tensormap(&p.tmap);
        for (int s = 0; s < kTbRing; ++s) mbar_init(&bars[s], 1);
        fence_barrier_init();
    }
    __syncthreads();

    uint32_t gplane = 0;   // planes this CTA has consumed so far (ring slot and phase)
    for (int item = blockIdx.x; item < p.nitems; item += gridDim.x) {
        const int txi = item % p.ntx;
        const int rest = item / p.ntx;
        const int tyi = rest % p.nty, tzi = rest / p.nty;
        const int x0 = txi * p.TX, y0 = tyi * p.TY, z0 = tzi * p.ZC;
        const int z1 = min(z0 + p.ZC, p.n[2]);
        const int NI = (z1 - z0) + 2 * k;       // input planes z0-k .. z1+k-1
        const int gx0 = x0 - p.XH, gy0 = y0 - K, gz0 = z0 - k;   // global coords of box (0, 0, plane 0)
        auto issue = [&](int j) {
            const uint32_t g = gplane + (uint32_t)j;
            uint64_t* bar = &bars[g % kTbRing];
            mbar_arrive_expect_tx(bar, p.box_bytes);
            tma_load_3d((void*)ring(g), &p.tmap, bar, gx0 + p.H, gy0 + p.H, gz0 + j + p.H);
        };
        if (tid == 0) {
            fence_proxy_async();
            issue(0);
            if (NI > 1) issue(1);
        }
        // per-thread constants: which of the block's cells lie outside the grid (Remove masks) and
        // whether it lies in the tile's interior (the stored outputs)
        int xout = 0, yout = 0;
#pragma unroll
        for (int c = 0; c < 4; ++c) xout |= (gx0 + cx + c < 0 || gx0 + cx + c >= p.n[0]) ? (1 << c) : 0;
#pragma unroll
        for (int r = 0; r < kTbRPT; ++r) yout |= (gy0 + cy + r < 0 || gy0 + cy + r >= p.n[1]) ? (1 << r) : 0;
        const bool own_out = act && cx >= p.XH && cx < p.XH + p.TX && cy >= K && cy < K + p.TY &&
                             gx0 + cx < p.n[0] && gy0 + cy < p.n[1];
        const bool full4 = gx0 + cx + 3 < p.n[0];

        // S[t-2][u]: level t's own-height plane (level t-1's cells at plane i - t, read from shared
        // memory for the fold) of the iterations with i mod 2 == u, t = 2 .. K.  The one read in the
        // previous iteration is this iteration's plane below (LO): its shared-memory buffer has been
        // overwritten by then.  Iterations run in pairs, so the set index is a compile-time constant and
        // nothing is copied between registers.  Level 1 reads its three planes from the input ring.
        float S[K - 1][2][kTbRPT][4];
        bool failed = false;
        auto iteration = [&](const int i, auto u_c) {
            constexpr int U = decltype(u_c)::value;
            if (tid == 0 && i + 2 < NI) {
                fence_proxy_async();
                issue(i + 2);
            }
            const uint32_t gi = gplane + (uint32_t)i;
            const bool ok = mbar_wait_bounded(&bars[gi % kTbRing], (gi / kTbRing) & 1u);
            if (!__syncthreads_and(ok)) {
                if (tid == 0) {
                    atomicOr(p.status, DEV_ERR_TIMEOUT);
                    for (int j = i; j < min(i + 3, NI); ++j) {
                        const uint32_t g = gplane + (uint32_t)j;
                        mbar_wait_bounded(&bars[g % kTbRing], (g / kTbRing) & 1u, 100000000ll);
                    }
                }
                failed = true;
                return;
            }
            float prev[kTbRPT][4];   // the plane the level below produced this iteration (this level's HI)
#pragma unroll
            for (int t = 1; t <= K; ++t) {
                if (!(i >= 2 * t - 1)) continue;   // uniform across the CTA
                const int pz = i - t;              // this level's plane (input-plane numbering)
                float LO[kTbRPT][4], HI[kTbRPT][4], UP[4], DN[4], EDGE[kTbRPT], LF[kTbRPT], RT[kTbRPT];
                float (&M)[kTbRPT][4] = S[t == 1 ? 0 : t - 2][t == 1 ? 0 : U];
                float M1[kTbRPT][4];
                float (&MM)[kTbRPT][4] = t == 1 ? M1 : M;
                if (i == 2 * t - 1) {
                    // the iteration before this level's first plane: read level t-1's plane below it
                    if (t >= 2) tb_own<float>(lvl(t - 1, pz & 1), BX, cx, cy, MM);
                    continue;
                }
                if (t == 1) {
                    const T* mid = ring(gplane + (uint32_t)pz);
                    tb_own<T>(mid, BX, cx, cy, MM);
                    tb_edges<T, Sh>(mid, BX, cx, cy, edge_off, UP, DN, EDGE);
                    if constexpr (TbTaps<Sh>::has(0, 0, -1)) tb_own<T>(ring(gplane + (uint32_t)pz - 1), BX, cx, cy, LO);
                    if constexpr (TbTaps<Sh>::has(0, 0, 1)) tb_own<T>(ring(gplane + (uint32_t)pz + 1), BX, cx, cy, HI);
                } else {
                    const float* mid = lvl(t - 1, pz & 1);
                    tb_own<float>(mid, BX, cx, cy, MM);
                    tb_edges<float, Sh>(mid, BX, cx, cy, edge_off, UP, DN, EDGE);
#pragma unroll
                    for (int r = 0; r < kTbRPT; ++r)
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            LO[r][c] = S[t - 2][1 - U][r][c];
                            HI[r][c] = prev[r][c];
                        }
                }
                tb_sides<Sh>(MM, EDGE, lane, LF, RT);
                float res[kTbRPT][4];
                if constexpr (TbPairOp<OpF>::kPair) tb_fold_block2<OpF, Sh>(MM, LO, HI, UP, DN, LF, RT, p, res);
                else tb_fold_block<OpF, Sh>(MM, LO, HI, UP, DN, LF, RT, p, res);
                const int gz = gz0 + pz;
                if (t < k) {
                    if (p.remove) {
                        const bool zo = gz < 0 || gz >= p.n[2];
#pragma unroll
                        for (int r = 0; r < kTbRPT; ++r)
#pragma unroll
                            for (int c = 0; c < 4; ++c)
                                if (zo || ((yout >> r) & 1) || ((xout >> c) & 1)) res[r][c] = p.padf;
                    }
                    if (!(std::is_same_v<T, float>) && !p.keep_f32) {
#pragma unroll
                        for (int r = 0; r < kTbRPT; ++r)
#pragma unroll
                            for (int c = 0; c < 4; ++c) res[r][c] = tb_widen<T>(tb_round<T>(res[r][c]));
                    }
                    if (act) {
                        float* out = lvl(t, pz & 1);
#pragma unroll
                        for (int r = 0; r < kTbRPT; ++r)
                            *(float4*)(out + (cy + r) * BX + cx) = make_float4(res[r][0], res[r][1], res[r][2], res[r][3]);
                    }
#pragma unroll
                    for (int r = 0; r < kTbRPT; ++r)
#pragma unroll
                        for (int c = 0; c < 4; ++c) prev[r][c] = res[r][c];
                } else if (own_out) {
                    T* drow = (T*)p.dst + (int64_t)gz * p.dstr2 + gx0 + cx;
#pragma unroll
                    for (int r = 0; r < kTbRPT; ++r) {
                        const int gy = gy0 + cy + r;
                        if (gy >= p.n[1]) break;
                        T o[4];
#pragma unroll
                        for (int c = 0; c < 4; ++c) {
                            if constexpr (std::is_same_v<T, __nv_bfloat16>) {
                                if (p.stochastic) {
                                    const uint64_t lin = (uint64_t)(gx0 + cx + c) +
                                                         (uint64_t)p.n[0] * ((uint64_t)gy + (uint64_t)p.n[1] * (uint64_t)gz);
                                    o[c] = tb_bf16_stochastic(res[r][c], lin, p.round_step);
                                    continue;
                                }
                            }
                            o[c] = tb_round<T>(res[r][c]);
                        }
                        T* d = drow + (int64_t)gy * p.dstr1;
                        if (full4) tb_st4<T>(d, o);
                        else
#pragma unroll
                            for (int c = 0; c < 4; ++c)
                                if (gx0 + cx + c < p.n[0]) d[c] = o[c];
                    }
                }
            }
            __syncthreads();
        };
        for (int i0 = 0; i0 < NI && !failed; i0 += 2) {
            iteration(i0, std::integral_constant<int, 0>{});
            if (failed || i0 + 1 >= NI) break;
            iteration(i0 + 1, std::integral_constant<int, 1>{});
        }
        if (failed) return;
        gplane += (uint32_t)NI;
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

using TbLaunch = cudaError_t (*)(const TB6Params&, int grid, int threads, size_t smem, cudaStream_t);

template <class T, class Op, class Sh, int K>
static cudaError_t tb6_launch(const TB6Params& p, int grid, int threads, size_t smem, cudaStream_t s) {
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    std::call_once(once, [&] {
        int dev = 0, optin = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        attr = cudaFuncSetAttribute(tb6_kernel<T, Op, Sh, K>, cudaFuncAttributeMaxDynamicSharedMemorySize, optin);
    });
    if (attr != cudaSuccess) return attr;
    tb6_kernel<T, Op, Sh, K><<<grid, threads, smem, s>>>(p);
    return cudaGetLastError();
}

// fn: passes of kTbK levels; fn8: passes of 8 levels (BFloat16 state in the STC_KEEP_F32 mode)
struct TbEntry { int dt, opv, shape; TbLaunch fn, fn8; };

using VN3 = Shape<STC_SHAPE_VONNEUMANN, 1, 3>;
using CR3 = Shape<STC_SHAPE_CROSS, 1, 3>;
using DiffBF = OpDiffuse<__nv_bfloat16, __nv_bfloat16, float>;
static const TbEntry kTbTable[] = {
    {STC_F32, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, &tb6_launch<float, OpDiffuse<float, float, float>, VN3, kTbK>, nullptr},
    {STC_BF16, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, &tb6_launch<__nv_bfloat16, DiffBF, VN3, kTbK>,
     &tb6_launch<__nv_bfloat16, DiffBF, VN3, kTbKMax>},
    {STC_F16, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, &tb6_launch<__half, OpDiffuse<__half, __half, float>, VN3, kTbK>, nullptr},
    {STC_F32, OPV_MEAN, STC_SHAPE_VONNEUMANN, &tb6_launch<float, OpMean<float, float, float>, VN3, kTbK>, nullptr},
    {STC_F32, OPV_SUM, STC_SHAPE_CROSS, &tb6_launch<float, OpSumF<float, float, float>, CR3, kTbK>, nullptr},
};

static CUtensorMapDataType tb_dtype(int dt) {
    return dt == STC_F32 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
           : dt == STC_BF16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT16;
}

static const TbEntry* tb_find(const stc_grid* a, const stc_stencil* st, const stc_op* op) {
    const int opv = op->code == STC_OP_DIFFUSE ? OPV_DIFFUSE : op->code == STC_OP_MEAN ? OPV_MEAN
                    : op->code == STC_OP_SUM ? OPV_SUM : -1;
    for (const TbEntry& e : kTbTable)
        if (e.dt == a->dtype && e.opv == opv && table_matches_shape(e.shape, 1, 3, st->offsets, st->len)) return &e;
    return nullptr;
}

// Levels per pass: 8 for BFloat16 state in the precision mode (half the stochastic roundings of 4, which
// measured 1.04e-2 max relative error on 512^3 x 200 diffusion against the 1e-2 target), else kTbK.
int tb3d_levels(int dtype, uint32_t flags) {
    return ((flags & STC_KEEP_F32) && dtype == STC_BF16) ? kTbKMax : kTbK;
}

bool tb3d_applies(const stc_grid* a, const stc_stencil* st, const stc_op* op, const stc_bc* bc) {
    if (a->ndims != 3 || st->ndims != 3 || st->radius != 1) return false;
    if (!(bc->boundary == STC_WRAP || bc->boundary == STC_REMOVE)) return false;
    if (!tb_find(a, st, op) || !tb_encoder()) return false;
    return true;
}

// Steps of the run taken by blocked passes of K steps: the largest multiple of K below nsteps; the rest
// (1 to K steps, so that the pair holds states n - 1 and n at the end) run as per-step maps on the pair.
static int64_t tb_blocked_steps(int64_t nsteps, int K) { return nsteps >= 1 ? (nsteps - 1) / K * K : 0; }

int tb3d_try_steps(const stc_grid* a, const stc_grid* b, const stc_stencil* st, const stc_op* op, const stc_bc* bc,
                   int64_t nsteps, int* src_is_b, cudaStream_t stream, DeviceCtx* ctx, uint32_t flags, int64_t* done) {
    *done = 0;
    const bool keep = (flags & STC_KEEP_F32) != 0 && (a->dtype == STC_BF16 || a->dtype == STC_F16);
    if (nsteps < 1) return STC_OK;
    // tuning / test override: STC_TBLOCK=0 disables the blocked path, =1 takes it for 16-bit state too
    const char* env = getenv("STC_TBLOCK");
    const bool disabled = env && env[0] == '0', forced = env && env[0] == '1';
    if (!tb3d_applies(a, st, op, bc) || disabled) return keep ? STC_ERR_UNSUPPORTED : STC_OK;
    if (!keep && nsteps < 8) return STC_OK;   // copies in and out would outweigh the saving
    // 16-bit state rounded every step: the per-step vector map moves half the bytes of Float32 and was
    // measured faster than the blocked kernel (711 against 557 Gcell/s on 512^3 x 200 BFloat16)
    if (!keep && !forced && a->dtype != STC_F32) return STC_OK;
    const int K = tb3d_levels(a->dtype, flags);
    const TbEntry* ent = tb_find(a, st, op);
    TbLaunch fn = K == kTbKMax ? ent->fn8 : ent->fn;
    if (!fn) return keep ? STC_ERR_UNSUPPORTED : STC_OK;
    const int es = dtype_size(a->dtype);
    const bool halo = bc->padding != STC_CONDITIONAL;
    int64_t n[3];
    for (int d = 0; d < 3; ++d) n[d] = a->size[d] - (halo ? 2 : 0);
    const int XH = std::max(K, 16 / es);   // tile's first column on a 16-byte boundary of the box
    const int H = XH;
    for (int d = 0; d < 3; ++d)
        if (n[d] < H || n[d] + 2 * H + 256 >= (1ll << 31)) return keep ? STC_ERR_UNSUPPORTED : STC_OK;

    // geometry: a tile of TX = 64 or 128 columns and the box height (rows a multiple of kTbRPT) with at
    // most 16 warps whose ring and level buffers fit, choosing the pair that computes the fewest box
    // cells per plane of the grid
    TB6Params p;
    memset(&p, 0, sizeof(p));
    p.XH = XH;
    p.H = H;
    const size_t smem_cap = (size_t)ctx->max_smem_optin;
    auto smem_for = [&](int BX, int BY, uint32_t* ring_off, uint32_t* ring_stride, uint32_t* lvl_off,
                        uint32_t* lvl_stride, uint32_t* bar_off) {
        const uint32_t slack = (uint32_t)((BX * es + 127) / 128 * 128);
        const uint32_t rs = (uint32_t)(((size_t)BX * BY * es + 127) / 128 * 128);
        const uint32_t ls = (uint32_t)(((size_t)BX * (BY + 2) * 4 + 127) / 128 * 128);
        *ring_off = slack;
        *ring_stride = rs;
        *lvl_off = slack + kTbRing * rs;
        *lvl_stride = ls;
        *bar_off = *lvl_off + 2 * (K - 1) * ls;
        return (size_t)*bar_off + 8 * kTbRing;
    };
    int best_by = 0, best_tx = 0;
    int64_t best_cost = INT64_MAX;
    for (int TX : {64, 128}) {
        const int BX = TX + 2 * XH;
        for (int BY = 2 * K + 8; BY <= 256; BY += kTbRPT) {
            uint32_t a0, a1, a2, a3, a4;
            if (smem_for(BX, BY, &a0, &a1, &a2, &a3, &a4) > smem_cap) break;
            const int threads = (BX / 4) * (BY / kTbRPT);
            if (threads > kTbMaxThreads) break;
            const int TY = BY - 2 * K;
            const int64_t cost = (n[0] + TX - 1) / TX * BX * ((n[1] + TY - 1) / TY * BY);
            if (cost < best_cost) {
                best_cost = cost;
                best_by = BY;
                best_tx = TX;
            }
        }
    }
    if (!best_by) return keep ? STC_ERR_UNSUPPORTED : STC_OK;
    p.TX = best_tx;
    p.BX = p.TX + 2 * XH;
    p.BY = best_by;
    p.TY = p.BY - 2 * K;
    const size_t smem = smem_for(p.BX, p.BY, &p.ring_off, &p.ring_stride, &p.lvl_off, &p.lvl_stride, &p.bar_off);
    const int threads = ((p.BX / 4) * (p.BY / kTbRPT) + 31) / 32 * 32;
    p.box_bytes = (uint32_t)((size_t)p.BX * p.BY * es);
    for (int d = 0; d < 3; ++d) p.n[d] = (int32_t)n[d];
    p.ntx = (int)((n[0] + p.TX - 1) / p.TX);
    p.nty = (int)((n[1] + p.TY - 1) / p.TY);
    // z chunks: the count whose waves of one CTA per SM (time ~ chunk planes + 2k) finish soonest
    {
        const int64_t xy = (int64_t)p.ntx * p.nty;
        int64_t best = INT64_MAX;
        int bz = 1;
        for (int c = 1; c <= std::max<int64_t>(1, n[2] / 8); ++c) {
            const int64_t zc = (n[2] + c - 1) / c;
            const int64_t waves = (xy * c + ctx->num_sms - 1) / ctx->num_sms;
            const int64_t cost = waves * (zc + 2 * K);
            if (cost < best) { best = cost; bz = c; }
        }
        p.ZC = (int)((n[2] + bz - 1) / bz);
        p.nzc = (int)((n[2] + p.ZC - 1) / p.ZC);
    }
    p.nitems = p.ntx * p.nty * p.nzc;
    const int grid = (int)std::min<int64_t>(p.nitems, ctx->num_sms);
    p.remove = bc->boundary == STC_REMOVE;
    {
        // padval in the storage type (as the reference's getneighbor returns it), widened
        const double pv = bc->padval;
        if (a->dtype == STC_F32) p.padf = (float)pv;
        else if (a->dtype == STC_BF16) { __nv_bfloat16 h = __float2bfloat16_rn((float)pv); p.padf = __bfloat162float(h); }
        else { __half h = __double2half(pv); p.padf = __half2float(h); }
    }
    p.keep_f32 = keep;
    p.stochastic = keep && a->dtype == STC_BF16;
    p.status = status_slot(ctx, stream).dev;
    p.L = st->len;
    p.alpha = op->alpha;
    p.rcp_f = (float)(1.0 / (double)st->len);
    p.fastdiv_f = op->code == STC_OP_MEAN ? (int)fastdiv_f_exact(st->len) : 0;
    p.Lf = (float)st->len;
    p.Ld = (double)st->len;
    p.alpha_f = (float)op->alpha;

    // the padded pair: rows of `pitch` elements, interior x = 0 on a 128-byte line
    const int64_t line = 128 / es;
    const int64_t lead = (H + line - 1) / line * line - H;   // unused elements before the ring
    const int64_t P0 = n[0] + 2 * H, P1 = n[1] + 2 * H, P2 = n[2] + 2 * H;
    const int64_t pitch = (lead + P0 + line - 1) / line * line;
    const size_t cells = (size_t)pitch * P1 * P2;
    char* mem = nullptr;
    bool cached = false;
    if (workspace_acquire(2 * cells * es + 256, stream, (void**)&mem, &cached) != STC_OK)
        return keep ? STC_ERR_CUDA : STC_OK;
    stc_grid pg[2];
    for (int i = 0; i < 2; ++i) {
        pg[i].ndims = 3;
        pg[i].dtype = a->dtype;
        pg[i].size[0] = P0;
        pg[i].size[1] = P1;
        pg[i].size[2] = P2;
        pg[i].stride[0] = 1;
        pg[i].stride[1] = pitch;
        pg[i].stride[2] = pitch * P1;
        pg[i].data = mem + (i * cells + lead) * es;
    }
    stc_bc hb = *bc;
    hb.padding = STC_HALO_OUT;
    const int64_t inner = H + H * pitch + H * pitch * P1;    // offset of logical (0, 0, 0) in a padded buffer
    const int64_t org_a = halo ? 1 + a->stride[1] + a->stride[2] : 0;
    const int64_t org_b = halo ? 1 + b->stride[1] + b->stride[2] : 0;
    const stc_grid* par[2] = {a, b};
    const int64_t org[2] = {org_a, org_b};
    int rc = launch_grid_copy(par[*src_is_b], org[*src_is_b], &pg[0], inner, n, stream);
    if (!rc && p.remove) rc = launch_halo_fill(&pg[0], H, &hb, stream);
    if (!rc && p.remove) rc = launch_halo_fill(&pg[1], H, &hb, stream);
    const int64_t blocked = tb_blocked_steps(nsteps, K);
    int cur = 0;
    int64_t step = 0;
    while (step < blocked && !rc) {
        if (!p.remove && (rc = launch_halo_fill(&pg[cur], H, &hb, stream))) break;
        step += K;
        p.round_step = (uint32_t)step;
        p.dst = (char*)pg[1 - cur].data + inner * es;
        p.dstr1 = pitch;
        p.dstr2 = pitch * P1;
        cuuint64_t gdim[3] = {(cuuint64_t)P0, (cuuint64_t)P1, (cuuint64_t)P2};
        cuuint64_t gstr[2] = {(cuuint64_t)(pitch * es), (cuuint64_t)(pitch * P1 * es)};
        cuuint32_t box[3] = {(cuuint32_t)p.BX, (cuuint32_t)p.BY, 1}, est[3] = {1, 1, 1};
        if (tb_encoder()(&p.tmap, tb_dtype(a->dtype), 3, pg[cur].data, gdim, gstr, box, est, CU_TENSOR_MAP_INTERLEAVE_NONE,
                         CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                         CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS) {
            rc = STC_ERR_UNSUPPORTED;
            break;
        }
        void* prof = prof_begin(stream);
        cudaError_t e = fn(p, grid, threads, smem, stream);
        prof_end(prof, stream, "tblock3d", 2.0 * es * n[0] * n[1] * n[2] * K, (double)n[0] * n[1] * n[2] * K);
        if (e != cudaSuccess) rc = cuda_fail(e);
        cur = 1 - cur;
    }
    // the remaining steps: per-step maps (K2 ring refresh, K1) on the pair seen as parents with a
    // one-cell Halo ring, each rounded to the storage type as a separate map is
    stc_grid view[2];
    for (int v = 0; v < 2; ++v) {
        view[v] = pg[v];
        view[v].data = (char*)pg[v].data + (inner - 1 - pitch - pitch * P1) * es;
        for (int d = 0; d < 3; ++d) view[v].size[d] = n[d] + 2;
    }
    for (; step < nsteps && !rc; ++step) {
        if ((rc = launch_halo_fill(&view[cur], 1, &hb, stream))) break;
        if ((rc = launch_map(&view[cur], &view[1 - cur], 1, st, op, &hb, stream, ctx))) break;
        cur = 1 - cur;
    }
    // state n to the parent the reference leaves it in, state n - 1 to the other
    const int res_b = (*src_is_b) ^ (int)(nsteps & 1);
    if (!rc) rc = launch_grid_copy(&pg[cur], inner, par[res_b], org[res_b], n, stream);
    if (!rc && nsteps > 1) rc = launch_grid_copy(&pg[1 - cur], inner, par[1 - res_b], org[1 - res_b], n, stream);
    workspace_release(mem, cached, stream);
    if (rc) return rc;
    *src_is_b = res_b;
    *done = nsteps;
    return STC_OK;
}

}  // namespace stc
