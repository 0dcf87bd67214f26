// map_kernel.cuh — K1, the gather-map kernel: dst[I] = f(stencil(src, I)) for every logical I.
//
// Replaces gatherstencil_kernel! (src/gatherstencil.jl:105-109) with stencil(A, I) (src/array.jl:22-30).
//
// Design (GB300):
//  * persistent CTAs walk output tiles; each tile's input box (tile + halo) is staged into shared
//    memory by TMA (cp.async.bulk.tensor, no multicast) through a multi-stage mbarrier pipeline, so
//    the next tiles stream in while the current one is reduced;
//  * boundary conditions live only in the loader: Halo padding reads the halo ring from memory,
//    Remove with a zero padval uses TMA's zero fill, and Wrap / Reflect / nonzero Remove patch the
//    out-of-range cells of edge tiles after the copy lands (src/array.jl:129-188);
//  * parents whose strides are not 16-byte multiples (e.g. a 4098-wide UInt8 halo parent) use a
//    cooperative load of the same box with the boundary mapping applied per element;
//  * the reduction folds over the neighbours in offset order.  The generic kernel reads the offset
//    table at run time; the shape-specialised kernels take the table as a compile-time constant and
//    stream the box along the slowest tiled axis, so every loaded value is reused from registers by
//    all outputs of the thread that need it, while keeping each output's fold order.
#pragma once

#include <cstring>
#include <type_traits>

#include "common.cuh"

namespace stc {

constexpr int kMapThreads = 256;
constexpr int kMapWarps = kMapThreads / 32;
constexpr int kMaxStages = 4;

struct MapParams {
    CUtensorMap tmap;          // source parent, valid when use_tma
    const void* src;           // source parent base
    void* dst;                 // destination parent base
    int64_t sst[3];            // source strides (elements; 0 beyond ndims)
    int64_t dstr[3];           // destination strides
    int64_t src_org;           // parent offset of logical (0,0,0)
    int64_t dst_org;
    int64_t n[3];              // logical size (1 beyond ndims)
    int64_t ntx, nty, ntz, ntiles;
    double padf;               // Remove padval in the source type (floats)
    int64_t padi;              // Remove padval (integers)
    double alpha;              // DIFFUSE
    int32_t hx[3];             // parent coordinate of logical 0 per axis (R for Halo padding)
    int32_t halo;              // halo ring present in memory
    int32_t boundary;
    int32_t ndims;
    int32_t rx, ry, rz;        // box halo per axis (largest |offset| along it)
    int32_t padl;              // shared-memory x index of the tile's first column
    int32_t tw, th, tz;        // tile extents (outputs)
    int32_t bw, bh, bd;        // box extents (inputs)
    int32_t tiles3d;           // 1: threads map (warp, slot) -> (y, z); 0: -> (y)
    int32_t use_tma;
    int32_t stages;
    int32_t fixup;             // edge tiles need patching after TMA (Wrap / Reflect / nonzero Remove)
    uint32_t box_bytes;
    uint32_t stage_bytes;
    int32_t* status;
    int32_t L;
    uint32_t birth, survive;
    float rcp_f;               // RN(1/L) in float, used when fastdiv_f (host-verified exact for this L)
    float Lf;                  // L and alpha pre-converted, so kernels never convert per cell
    double Ld;
    float alpha_f;
    int32_t fastdiv_f;
    int8_t off[STC_MAX_LEN][3];
    float wf[STC_MAX_LEN];
    double w[STC_MAX_LEN];
};

// ---------------------------------------------------------------------------- reductions
// Each op: Acc type; first(v) = Base.reduce_first; step(a, v, k); finish(a, centre).
// KDOT starts from zero and steps every term (src/stencils/kernel.jl:37-43).

// Correctly rounded a / L with L a small positive integer.
// Float32: q = RN(a*r), e = a - q*L (exact by FMA), q' = RN(q + e*r) with r = RN(1/L).  The host enables
// this only after checking, for this L, that q' equals the correctly rounded quotient for every
// mantissa of one binade; the result pattern repeats in every binade while the intermediates stay
// normal, hence the |a| >= 2^-90 guard.  Otherwise the IEEE division is used.
template <class P> __device__ __forceinline__ float div_by_len(float a, const P& p) {
    if (p.fastdiv_f && fabsf(a) >= 0x1p-90f && fabsf(a) <= 3.0e38f) {
        const float q = __fmul_rn(a, p.rcp_f);
        const float e = __fmaf_rn(-q, p.Lf, a);
        return __fmaf_rn(e, p.rcp_f, q);
    }
    return __fdiv_rn(a, p.Lf);
}
// Float64 uses the IEEE division: on GB300 every FP64 instruction is costly, and a verified FMA
// quotient needs more of them than __ddiv_rn.
template <class P> __device__ __forceinline__ double div_by_len(double a, const P& p) {
    return __ddiv_rn(a, p.Ld);
}

// The mean's Float32 quotient without a per-output range test: true if the FMA-corrected quotient of a
// (div_by_len's fast branch) is exact, i.e. the host verified it for this L and a is in [2^-90, 3e38].
template <class P> __device__ __forceinline__ bool fastdiv_in_range(float a, const P& p) {
    return p.fastdiv_f && fabsf(a) >= 0x1p-90f && fabsf(a) <= 3.0e38f;
}
template <class P> __device__ __forceinline__ float fastdiv_quotient(float a, const P& p) {
    const float q = __fmul_rn(a, p.rcp_f);
    const float e = __fmaf_rn(-q, p.Lf, a);
    return __fmaf_rn(e, p.rcp_f, q);
}

// Correctly rounded a / LC for a compile-time 2 <= LC <= 512, in integer arithmetic (schoolbook
// binary division with guard and sticky bits, IEEE 754 round to nearest even): the 53-bit significand
// shifted left by 11 is divided by the constant (a multiply-high, no division instruction), the quotient
// keeps at least 55 bits, its low bits and the remainder give the round and sticky bits.  Zero,
// subnormal, infinite and NaN inputs and subnormal results use the IEEE division.  On GB300 this costs a
// few dozen integer instructions instead of the FP64 instructions of a division.
template <int LC>
__device__ __forceinline__ double div_exact_const(double a) {
    static_assert(LC >= 2 && LC <= 512, "constant divisor range");
    const unsigned long long b = (unsigned long long)__double_as_longlong(a);
    const unsigned ex = (unsigned)(b >> 52) & 0x7ffu;
    if (ex == 0u || ex == 0x7ffu) return __ddiv_rn(a, (double)LC);
    const unsigned long long N = ((b & 0xfffffffffffffull) | (1ull << 52)) << 11;
    const unsigned long long Q = N / (unsigned long long)LC;
    const unsigned long long rem = N - Q * (unsigned long long)LC;
    const int t = 11 - __clzll((long long)Q);          // bits of Q beyond 53 (>= 2)
    unsigned long long mant = Q >> t;
    const unsigned long long low = Q & ((1ull << t) - 1ull);
    const bool rnd = ((low >> (t - 1)) & 1ull) != 0ull;
    const bool sticky = (low & ((1ull << (t - 1)) - 1ull)) != 0ull || rem != 0ull;
    int E = (int)ex - 1023 + t - 11;                    // exponent of mant / 2^52
    if (rnd && (sticky || (mant & 1ull))) mant += 1ull;
    if (mant == (1ull << 53)) {
        mant >>= 1;
        E += 1;
    }
    if (E + 1023 <= 0) return __ddiv_rn(a, (double)LC);
    return __longlong_as_double(
        (long long)((b & (1ull << 63)) | ((unsigned long long)(E + 1023) << 52) | (mant - (1ull << 52))));
}

template <class Tin, class Tout, class Acc> struct OpMean {
    static constexpr bool kZeroInit = false, kNeedsCentre = false;
    using A = Acc;
    __device__ static A first(Tin v, int) { return conv(v); }
    template <class P> __device__ static A step(A a, Tin v, int, const P&) { return add(a, conv(v)); }
    template <class P> __device__ static Tout finish(A a, Tin, const P& p) {
        if constexpr (sizeof(A) == 8) return from_f64<Tout>(div_by_len(a, p));
        else return from_f32<Tout>(div_by_len(a, p));
    }
    // finish with the stencil length known at compile time (shape-specialised kernels)
    template <int LC, class P> __device__ static Tout finish_c(A a, Tin c, const P& p) {
        if constexpr (sizeof(A) == 8 && LC >= 2 && LC <= 512) return from_f64<Tout>(div_exact_const<LC>(a));
        else return finish(a, c, p);
    }
    __device__ static A conv(Tin v) {
        if constexpr (sizeof(A) == 8) return cvt_d(v); else return cvt_f(v);
    }
    __device__ static A add(A a, A b) {
        if constexpr (sizeof(A) == 8) return __dadd_rn(a, b); else return __fadd_rn(a, b);
    }
};

template <class Tin, class Tout, class Acc> struct OpSumF {
    static constexpr bool kZeroInit = false, kNeedsCentre = false;
    using A = Acc;
    __device__ static A first(Tin v, int) { return OpMean<Tin, Tout, Acc>::conv(v); }
    template <class P> __device__ static A step(A a, Tin v, int, const P&) {
        return OpMean<Tin, Tout, Acc>::add(a, OpMean<Tin, Tout, Acc>::conv(v));
    }
    template <class P> __device__ static Tout finish(A a, Tin, const P&) {
        if constexpr (sizeof(A) == 8) return from_f64<Tout>(a); else return from_f32<Tout>(a);
    }
};

// integer sum: wraps at the accumulator's width (UInt8 sums stay UInt8; Bool widens to Int64)
template <class Tin, class Tout, int ACC_DT> struct OpSumI {
    static constexpr bool kZeroInit = false, kNeedsCentre = false;
    using A = int64_t;
    __device__ static A first(Tin v, int) { return cvt_i(v); }
    template <class P> __device__ static A step(A a, Tin v, int, const P&) {
        return wrap_int<ACC_DT>((int64_t)((uint64_t)a + (uint64_t)cvt_i(v)));
    }
    template <class P> __device__ static Tout finish(A a, Tin, const P&) { return (Tout)a; }
};

// kernelproduct in f64: product and sum rounded separately (no FMA), as the reference
template <class Tin, class Tout> struct OpKdotD {
    static constexpr bool kZeroInit = true, kNeedsCentre = false;
    using A = double;
    __device__ static A first(Tin v, int) { return 0.0; }
    template <class P> __device__ static A step(A a, Tin v, int k, const P& p) {
        return __dadd_rn(a, __dmul_rn(cvt_d(v), p.w[k]));
    }
    template <class P> __device__ static Tout finish(A a, Tin, const P&) { return from_f64<Tout>(a); }
};

// kernelproduct with f32 accumulation: fused multiply-add (tolerance path, error vs FP64 stated)
template <class Tin, class Tout> struct OpKdotF {
    static constexpr bool kZeroInit = true, kNeedsCentre = false;
    using A = float;
    __device__ static A first(Tin v, int) { return 0.0f; }
    template <class P> __device__ static A step(A a, Tin v, int k, const P& p) { return fmaf(cvt_f(v), p.wf[k], a); }
    template <class P> __device__ static Tout finish(A a, Tin, const P&) { return from_f32<Tout>(a); }
};

template <class Tin, class Tout, class Acc, bool MAX> struct OpMinMaxF {
    static constexpr bool kZeroInit = false, kNeedsCentre = false;
    using A = Acc;
    __device__ static A first(Tin v, int) { return OpMean<Tin, Tout, Acc>::conv(v); }
    template <class P> __device__ static A step(A a, Tin v, int, const P&) {
        A b = OpMean<Tin, Tout, Acc>::conv(v);
        return MAX ? jl_max(a, b) : jl_min(a, b);
    }
    template <class P> __device__ static Tout finish(A a, Tin, const P&) {
        if constexpr (sizeof(A) == 8) return from_f64<Tout>(a); else return from_f32<Tout>(a);
    }
};

template <class Tin, class Tout, bool MAX> struct OpMinMaxI {
    static constexpr bool kZeroInit = false, kNeedsCentre = false;
    using A = int64_t;
    __device__ static A first(Tin v, int) { return cvt_i(v); }
    template <class P> __device__ static A step(A a, Tin v, int, const P&) {
        A b = cvt_i(v);
        return MAX ? (b > a ? b : a) : (b < a ? b : a);
    }
    template <class P> __device__ static Tout finish(A a, Tin, const P&) { return (Tout)a; }
};

template <class Tin, class Tout> struct OpLife {
    static constexpr bool kZeroInit = false, kNeedsCentre = true;
    using A = int32_t;
    __device__ static A first(Tin v, int) { return v != (Tin)0; }
    template <class P> __device__ static A step(A a, Tin v, int, const P&) { return a + (v != (Tin)0); }
    template <class P> __device__ static Tout finish(A a, Tin c, const P& p) {
        uint32_t mask = (c != (Tin)0) ? p.survive : p.birth;
        return (Tout)((mask >> a) & 1u);
    }
};

// c + alpha * (sum(hood) - L*c), every operation rounded separately
template <class Tin, class Tout, class Acc> struct OpDiffuse {
    static constexpr bool kZeroInit = false, kNeedsCentre = true;
    using A = Acc;
    __device__ static A first(Tin v, int k) { return OpMean<Tin, Tout, Acc>::conv(v); }
    template <class P> __device__ static A step(A a, Tin v, int k, const P& p) {
        return OpMean<Tin, Tout, Acc>::add(a, OpMean<Tin, Tout, Acc>::conv(v));
    }
    template <class P> __device__ static Tout finish(A s, Tin cv, const P& p) {
        if constexpr (sizeof(A) == 8) {
            double c = cvt_d(cv);
            double t = __dmul_rn(p.Ld, c);
            t = __dsub_rn(s, t);
            t = __dmul_rn(p.alpha, t);
            return from_f64<Tout>(__dadd_rn(c, t));
        } else {
            float c = cvt_f(cv);
            float t = __fmul_rn(p.Lf, c);
            t = __fsub_rn(s, t);
            t = __fmul_rn(p.alpha_f, t);
            return from_f32<Tout>(__fadd_rn(c, t));
        }
    }
};

// ---------------------------------------------------------------------------- shapes
struct Off3 { int x, y, z; };
template <int MAXL> struct OffTable { int len; Off3 o[MAXL]; };

constexpr int ipow(int b, int e) { return e == 0 ? 1 : b * ipow(b, e - 1); }

// The offsets Stencils.jl generates, in its column-major order (axis 0 fastest):
// Window (src/stencils/window.jl:4-7, N<=2), Moore (moore.jl:5-18), VonNeumann (vonneumman.jl:5-15),
// Circle (shapes.jl:58-67; sqrt(s) < R+0.5 <=> s <= R^2+R for integer s), Cross (shapes.jl:2-10).
template <int KIND, int R, int N>
constexpr OffTable<ipow(2 * R + 1, N)> make_shape() {
    OffTable<ipow(2 * R + 1, N)> t{};
    t.len = 0;
    const int zr = N >= 3 ? R : 0, yr = N >= 2 ? R : 0;
    for (int z = -zr; z <= zr; ++z)
        for (int y = -yr; y <= yr; ++y)
            for (int x = -R; x <= R; ++x) {
                const int m = (x < 0 ? -x : x) + (y < 0 ? -y : y) + (z < 0 ? -z : z);
                const int s2 = x * x + y * y + z * z;
                const int zeros = (x == 0) + (N >= 2 && y == 0) + (N >= 3 && z == 0);
                bool in = false;
                if (KIND == STC_SHAPE_WINDOW) in = true;
                else if (KIND == STC_SHAPE_MOORE) in = m != 0;
                else if (KIND == STC_SHAPE_VONNEUMANN) in = m >= 1 && m <= R;
                else if (KIND == STC_SHAPE_CIRCLE) in = s2 <= R * R + R;
                else if (KIND == STC_SHAPE_CROSS) in = zeros >= N - 1;
                if (in) t.o[t.len++] = Off3{x, y, z};
            }
    return t;
}

template <int KIND, int R, int N> struct Shape {
    static constexpr int kKind = KIND, kR = R, kN = N;
    static constexpr auto table = make_shape<KIND, R, N>();
    static constexpr int L = table.len;
};

// ---------------------------------------------------------------------------- loaders
__device__ __forceinline__ int64_t bound_axis(int boundary, int64_t i, int64_t s) {
    if (boundary == STC_WRAP) return i < 0 ? i + s : (i >= s ? i - s : i);
    // Reflect: 1-based 2-i / 2s-i, i.e. 0-based -j / 2s-2-j
    return i < 0 ? -i : (i >= s ? 2 * s - 2 - i : i);
}

template <class Tin> __device__ __forceinline__ Tin padval_as(const MapParams& p);
template <> __device__ __forceinline__ double padval_as<double>(const MapParams& p) { return p.padf; }
template <> __device__ __forceinline__ float padval_as<float>(const MapParams& p) { return (float)p.padf; }
template <> __device__ __forceinline__ __nv_bfloat16 padval_as<__nv_bfloat16>(const MapParams& p) {
    return __float2bfloat16_rn((float)p.padf);
}
template <> __device__ __forceinline__ __half padval_as<__half>(const MapParams& p) {
    return __double2half(p.padf);
}
template <> __device__ __forceinline__ uint8_t padval_as<uint8_t>(const MapParams& p) { return (uint8_t)p.padi; }
template <> __device__ __forceinline__ int32_t padval_as<int32_t>(const MapParams& p) {
    return (int32_t)(uint32_t)(uint64_t)p.padi;
}
template <> __device__ __forceinline__ int64_t padval_as<int64_t>(const MapParams& p) { return p.padi; }

// Value of logical cell (x, y, z) for cells that may lie outside [0, n): the Conditional rules.
template <class Tin>
__device__ __forceinline__ Tin load_bounded(const MapParams& p, int64_t x, int64_t y, int64_t z) {
    const Tin* src = (const Tin*)p.src;
    if (p.halo) return src[p.src_org + x + y * p.sst[1] + z * p.sst[2]];
    const bool in = x >= 0 && x < p.n[0] && y >= 0 && y < p.n[1] && z >= 0 && z < p.n[2];
    if (!in) {
        if (p.boundary == STC_REMOVE) return padval_as<Tin>(p);
        x = bound_axis(p.boundary, x, p.n[0]);
        y = bound_axis(p.boundary, y, p.n[1]);
        z = bound_axis(p.boundary, z, p.n[2]);
    }
    return src[p.src_org + x + y * p.sst[1] + z * p.sst[2]];
}

struct TileOrigin { int64_t x0, y0, z0; };

// tile counts per axis and in total stay below 2^31 (axes are < 2^31 cells), so 32-bit math suffices
__device__ __forceinline__ TileOrigin tile_origin(const MapParams& p, int64_t t) {
    TileOrigin o;
    const uint32_t ti = (uint32_t)t, ntx = (uint32_t)p.ntx, nty = (uint32_t)p.nty;
    const uint32_t r = ti / ntx;
    o.x0 = (int64_t)(ti - r * ntx) * p.tw;
    const uint32_t rz = r / nty;
    o.y0 = (int64_t)(r - rz * nty) * p.th;
    o.z0 = (int64_t)rz * p.tz;
    return o;
}

// Needed input region of a tile (clipped at the array end for ragged tiles), in logical coords.
struct Region { int64_t xa, xb, ya, yb, za, zb; };
__device__ __forceinline__ Region needed_region(const MapParams& p, const TileOrigin& o) {
    Region g;
    g.xa = o.x0 - p.rx; g.xb = min(o.x0 + p.tw, p.n[0]) + p.rx;
    g.ya = o.y0 - p.ry; g.yb = min(o.y0 + p.th, p.n[1]) + p.ry;
    g.za = o.z0 - p.rz; g.zb = min(o.z0 + p.tz, p.n[2]) + p.rz;
    return g;
}

__device__ __forceinline__ bool region_inside(const MapParams& p, const Region& g) {
    return g.xa >= 0 && g.xb <= p.n[0] && g.ya >= 0 && g.yb <= p.n[1] && g.za >= 0 && g.zb <= p.n[2];
}

// smem index of logical (x, y, z) for a tile at origin o
__device__ __forceinline__ int box_index(const MapParams& p, const TileOrigin& o, int64_t x, int64_t y,
                                         int64_t z) {
    return ((int)(z - o.z0 + p.rz) * p.bh + (int)(y - o.y0 + p.ry)) * p.bw + (int)(x - o.x0 + p.padl);
}

// Cooperative load of the needed region, one warp per box row.
template <class Tin>
__device__ void load_region(const MapParams& p, const TileOrigin& o, Tin* box) {
    const Region g = needed_region(p, o);
    const int wy = (int)(g.yb - g.ya), wz = (int)(g.zb - g.za);
    const int nrows = wy * wz;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const Tin* src = (const Tin*)p.src;
    for (int row = warp; row < nrows; row += nwarps) {
        const int64_t y = g.ya + row % wy, z = g.za + row / wy;
        Tin* brow = box + ((int)(z - o.z0 + p.rz) * p.bh + (int)(y - o.y0 + p.ry)) * p.bw + p.padl;
        const bool row_in = y >= 0 && y < p.n[1] && z >= 0 && z < p.n[2];
        if (p.halo || (row_in && g.xa >= 0 && g.xb <= p.n[0])) {
            // the whole row lies in memory: straight copy
            const Tin* srow = src + p.src_org + y * p.sst[1] + z * p.sst[2];
            for (int64_t x = g.xa + lane; x < g.xb; x += 32) brow[x - o.x0] = srow[x];
            continue;
        }
        for (int64_t x = g.xa + lane; x < g.xb; x += 32) brow[x - o.x0] = load_bounded<Tin>(p, x, y, z);
    }
}

// Patch of an edge tile after its TMA copy: only the needed cells outside [0, n) are written
// (Conditional rules), so the work is proportional to the outside cells.  Whole rows whose y or z
// lies outside: a warp per row.  Rows inside in y and z: only their x-halo cells beyond either end,
// one cell per thread, so those loads are all in flight together.
template <class Tin>
__device__ void patch_outside(const MapParams& p, const TileOrigin& o, Tin* box) {
    const Region g = needed_region(p, o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int wy = (int)(g.yb - g.ya), wz = (int)(g.zb - g.za);
    // rows with y inside, per plane: y in [yi0, yi1)
    const int64_t yi0 = max(g.ya, (int64_t)0), yi1 = min(g.yb, p.n[1]);
    const int nyi = (int)max((int64_t)0, yi1 - yi0);
    const int ylo = (int)(yi0 - g.ya);               // rows below 0 (or every row when none is inside)
    for (int zi = 0; zi < wz; ++zi) {
        const int64_t z = g.za + zi;
        const bool zin = z >= 0 && z < p.n[2];
        const int nout = zin ? wy - nyi : wy;        // rows of this plane to load whole
        for (int j = warp; j < nout; j += nwarps) {
            const int64_t y = zin ? (j < ylo ? g.ya + j : yi1 + (j - ylo)) : g.ya + j;
            Tin* brow = box + ((int)(z - o.z0 + p.rz) * p.bh + (int)(y - o.y0 + p.ry)) * p.bw + p.padl;
            for (int64_t x = g.xa + lane; x < g.xb; x += 32) brow[x - o.x0] = load_bounded<Tin>(p, x, y, z);
        }
    }
    // x-halo cells of the rows inside in y and z: [xa, 0) on the left, [n0, xb) on the right
    const int xl = (int)max((int64_t)0, min(g.xb, (int64_t)0) - g.xa);
    const int xr = (int)max((int64_t)0, g.xb - max(g.xa, p.n[0]));
    const int nx = xl + xr;
    if (nx == 0 || nyi == 0) return;
    const int64_t zi0 = max(g.za, (int64_t)0), zi1 = min(g.zb, p.n[2]);
    const int nzi = (int)max((int64_t)0, zi1 - zi0);
    const int items = nyi * nzi * nx;
    for (int it = threadIdx.x; it < items; it += blockDim.x) {
        const int row = it / nx, c = it - row * nx;
        const int ry = row % nyi, rz = row / nyi;
        const int64_t y = yi0 + ry, z = zi0 + rz;
        const int64_t x = c < xl ? g.xa + c : p.n[0] + (c - xl);
        box[box_index(p, o, x, y, z)] = load_bounded<Tin>(p, x, y, z);
    }
}

__device__ __forceinline__ void issue_tile_tma(const MapParams& p, const TileOrigin& o, void* box,
                                               uint64_t* bar) {
    const int cx = (int)(o.x0 + p.hx[0] - p.padl);
    const int cy = (int)(o.y0 + p.hx[1] - p.ry);
    const int cz = (int)(o.z0 + p.hx[2] - p.rz);
    mbar_arrive_expect_tx(bar, p.box_bytes);
    if (p.ndims == 1) tma_load_1d(box, &p.tmap, bar, cx);
    else if (p.ndims == 2) tma_load_2d(box, &p.tmap, bar, cx, cy);
    else tma_load_3d(box, &p.tmap, bar, cx, cy, cz);
}

__device__ __forceinline__ void report(const MapParams& p, int code) {
    if (p.status) atomicOr(p.status, code);
}

// ---------------------------------------------------------------------------- compute: generic
// Thread owns XT columns (lane + 32 i) and VS slots; slot s is row warp*VS + s (2D tiles) or
// (row warp, plane s) (3D tiles).  Each output folds over the run-time offset table in table order.
// The table loop is outermost: the XT x VS folds advance together as independent chains, and each
// offset's box displacement is formed once per thread.  Outputs past the grid's edge are folded too
// (every slot and column of the tile lies inside the box, whatever the grid's extent) and not stored.
template <class Tin, class Tout, class Op, int XT, int VS>
__device__ __forceinline__ void compute_generic(const MapParams& p, const TileOrigin& o, const Tin* box) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    Tout* dst = (Tout*)p.dst;
    const Tin* c[VS];
#pragma unroll
    for (int s = 0; s < VS; ++s) {
        const int ly = p.tiles3d ? warp : warp * VS + s;
        const int lz = p.tiles3d ? s : 0;
        c[s] = box + ((lz + p.rz) * p.bh + (ly + p.ry)) * p.bw + (lane + p.padl);
    }
#ifdef STC_DEBUG_BOUNDS
    {
        // every read of this thread lies within the staged box (centre and every offset, all columns)
        int dmin = 0, dmax = 0;
        for (int k = 0; k < p.L; ++k) {
            const int d = (p.off[k][2] * p.bh + p.off[k][1]) * p.bw + p.off[k][0];
            dmin = min(dmin, d);
            dmax = max(dmax, d);
        }
        const int64_t n = p.box_bytes / sizeof(Tin);
        bool bad = false;
        for (int s = 0; s < VS; ++s) {
            const int64_t b = c[s] - box;
            bad = bad || !STC_IN_BOUNDS(b + dmin, n, p.status) || !STC_IN_BOUNDS(b + 32 * (XT - 1) + dmax, n, p.status);
        }
        if (__any_sync(0xffffffffu, bad)) return;   // the whole warp: the finish below votes across it
    }
#endif
    typename Op::A a[VS][XT];
    int k0 = 0;
    if constexpr (Op::kZeroInit) {
#pragma unroll
        for (int s = 0; s < VS; ++s)
#pragma unroll
            for (int i = 0; i < XT; ++i) a[s][i] = Op::first(c[s][32 * i], 0);
    } else {
        const int d = (p.off[0][2] * p.bh + p.off[0][1]) * p.bw + p.off[0][0];
#pragma unroll
        for (int s = 0; s < VS; ++s)
#pragma unroll
            for (int i = 0; i < XT; ++i) a[s][i] = Op::first(c[s][32 * i + d], 0);
        k0 = 1;
    }
    for (int k = k0; k < p.L; ++k) {
        const int d = (p.off[k][2] * p.bh + p.off[k][1]) * p.bw + p.off[k][0];
#pragma unroll
        for (int s = 0; s < VS; ++s)
#pragma unroll
            for (int i = 0; i < XT; ++i) a[s][i] = Op::step(a[s][i], c[s][32 * i + d], k, p);
    }
    const int nvx = (int)min((int64_t)p.tw, p.n[0] - o.x0);
#pragma unroll
    for (int s = 0; s < VS; ++s) {
        const int ly = p.tiles3d ? warp : warp * VS + s;
        const int lz = p.tiles3d ? s : 0;
        const int64_t y = o.y0 + ly, z = o.z0 + lz;
        if (y >= p.n[1] || z >= p.n[2]) continue;
        Tout* drow = dst + p.dst_org + y * p.dstr[1] + z * p.dstr[2] + o.x0;
#pragma unroll
        for (int i = 0; i < XT; ++i) {
            const int lx = lane + 32 * i;
            if (lx < nvx) drow[lx] = Op::finish(a[s][i], c[s][32 * i], p);
        }
    }
}

// ---------------------------------------------------------------------------- compute: specialised
// Register-rotation stream along the slowest tiled axis (y for 2D shapes, z for 3D shapes).  The
// thread owns XT columns (lane + 32 i) and VS consecutive outputs along the stream axis.  Input rows
// r = 0 .. VS + 2R - 1 are visited once each, in increasing order; row r feeds the outputs
// s = r - q for q = 0 .. D-1 (D = 2R+1, q = offset row + R).  Output s lives in accumulator slot
// s mod D.  When the whole stream is small (rows x offsets) it is unrolled completely, so every
// slot, bound and address offset is a compile-time constant; otherwise the row loop is a run-time
// loop unrolled by D, which keeps slots, offsets and weights constant.  Because rows ascend and the
// generated tables are sorted by (z, y, x), each output folds its neighbours in table order; it is
// finished and stored right after its last row.
template <class Tin, class Tout, class Op, class Sh, int XT, int VS>
__device__ __forceinline__ void compute_shape(const MapParams& p, const TileOrigin& o, const Tin* box) {
    constexpr int N = Sh::kN, R = Sh::kR, L = Sh::L;
    constexpr int D = 2 * R + 1;
    constexpr int RY = (N == 3) ? R : 0;    // in-plane y halo for 3D shapes
    constexpr int NROW = VS + 2 * R;
    constexpr bool FULL = NROW * L <= 600;
    constexpr auto T = Sh::table;
    static_assert(((N == 3) ? T.o[0].z : T.o[0].y) == -R, "tables start at the lowest stream offset");
    using A = typename Op::A;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    A acc[XT][D];
    Tin ctr[XT][D];
#pragma unroll
    for (int i = 0; i < XT; ++i)
#pragma unroll
        for (int q = 0; q < D; ++q) { acc[i][q] = A(0); ctr[i][q] = Tin(0); }
    // box element (row r, in-plane row offset yy - RY, column lane + 32 i + xx - R) is
    // bb[r * sr + yy * p.bw + xx + 32 i]
    const int sr = (N == 3) ? p.bh * p.bw : p.bw;
    const Tin* bb = box + ((N == 3) ? (warp + p.ry - RY) * p.bw : p.rz * p.bh * p.bw + warp * VS * p.bw) + lane + p.padl - R;
#ifdef STC_DEBUG_BOUNDS
    {
        // the first and the last element this thread reads lie within the staged box (the whole warp leaves
        // together if one lane fails: the fold below votes across the warp)
        const int64_t n = p.box_bytes / sizeof(Tin), b = bb - box;
        const bool bad = !STC_IN_BOUNDS(b, n, p.status) ||
                         !STC_IN_BOUNDS(b + (NROW - 1) * sr + 2 * RY * p.bw + (D - 1) + 32 * (XT - 1), n, p.status);
        if (__any_sync(0xffffffffu, bad)) return;
    }
#endif
    // tile-local extents that hold real outputs (ragged last tiles)
    const int nvx = (int)min((int64_t)p.tw, p.n[0] - o.x0);
    const int nvs = (N == 3) ? (int)min((int64_t)VS, p.n[2] - o.z0) : (int)min((int64_t)VS, p.n[1] - o.y0 - warp * VS);
    const bool row_ok = (N == 3) ? (o.y0 + warp < p.n[1]) : true;
    // output s of this thread is dbase[s * dstep + lane + 32 i]
    Tout* dbase = (Tout*)p.dst + p.dst_org + o.x0 + lane +
                  ((N == 3) ? (o.y0 + warp) * p.dstr[1] + o.z0 * p.dstr[2] : (o.y0 + warp * VS) * p.dstr[1]);
    const int64_t dstep = (N == 3) ? p.dstr[2] : p.dstr[1];
    auto row = [&](const int r, const int u) {
        Tin v[XT][2 * RY + 1][D];
#pragma unroll
        for (int i = 0; i < XT; ++i)
#pragma unroll
            for (int yy = 0; yy < 2 * RY + 1; ++yy)
#pragma unroll
                for (int xx = 0; xx < D; ++xx) v[i][yy][xx] = bb[r * sr + yy * p.bw + xx + 32 * i];
#pragma unroll
        for (int q = 0; q < D; ++q) {
            const int sidx = r - q;               // output fed by this row at offset row q - R
            if (sidx < 0 || sidx >= VS) continue;
            const int slot = ((u - q) % D + D) % D;   // == sidx mod D (r - u is a multiple of D)
            if (Op::kZeroInit && q == 0) {
#pragma unroll
                for (int i = 0; i < XT; ++i) acc[i][slot] = Op::first(Tin(0), 0);
            }
#pragma unroll
            for (int k = 0; k < L; ++k) {
                const int ko = (N == 3) ? T.o[k].z : T.o[k].y;
                if (ko != q - R) continue;
                const int oy = (N == 3) ? T.o[k].y : 0;
#pragma unroll
                for (int i = 0; i < XT; ++i) {
                    const Tin val = v[i][oy + RY][T.o[k].x + R];
                    if (!Op::kZeroInit && k == 0) acc[i][slot] = Op::first(val, 0);
                    else acc[i][slot] = Op::step(acc[i][slot], val, k, p);
                }
            }
            if (Op::kNeedsCentre && q == R) {
#pragma unroll
                for (int i = 0; i < XT; ++i) ctr[i][slot] = v[i][RY][R];
            }
            if (q == D - 1 && sidx < nvs && row_ok) {
                // last row of output sidx: finish and store
                Tout* drow = dbase + sidx * dstep;
#pragma unroll
                for (int i = 0; i < XT; ++i) {
                    if (lane + 32 * i < nvx) {
                        if constexpr (std::is_same_v<Op, OpMean<Tin, Tout, A>>)
                            drow[32 * i] = Op::template finish_c<L>(acc[i][slot], ctr[i][slot], p);
                        else
                            drow[32 * i] = Op::finish(acc[i][slot], ctr[i][slot], p);
                    }
                }
            }
        }
    };
    if constexpr (FULL) {
#pragma unroll
        for (int r = 0; r < NROW; ++r) row(r, r % D);
    } else {
        for (int r0 = 0; r0 < NROW; r0 += D) {
#pragma unroll
            for (int u = 0; u < D; ++u) {
                const int r = r0 + u;
                if (r >= NROW) break;
                row(r, u);
            }
        }
    }
}

// ---------------------------------------------------------------------------- compute: vector columns
// Fold type of the vector path.  A 16-bit float source accumulated in Float32 is widened once per
// loaded element (exact), and the op is the same op over Float32 inputs: for these ops
// step(a, v) == step_f32(a, float(v)) and finish(a, c) == finish_f32(a, float(c)), so every output is
// bit-identical to the one-column path.
template <class Op> struct Widen { using type = Op; static constexpr bool kWide = false; };
#define STC_WIDEN3(OPT)                                                                                    \
    template <class Tout> struct Widen<OPT<__nv_bfloat16, Tout, float>> { using type = OPT<float, Tout, float>; static constexpr bool kWide = true; }; \
    template <class Tout> struct Widen<OPT<__half, Tout, float>> { using type = OPT<float, Tout, float>; static constexpr bool kWide = true; };
STC_WIDEN3(OpMean)
STC_WIDEN3(OpSumF)
STC_WIDEN3(OpDiffuse)
#undef STC_WIDEN3
template <class Tout> struct Widen<OpKdotF<__nv_bfloat16, Tout>> { using type = OpKdotF<float, Tout>; static constexpr bool kWide = true; };
template <class Tout> struct Widen<OpKdotF<__half, Tout>> { using type = OpKdotF<float, Tout>; static constexpr bool kWide = true; };
template <class Tout, bool MAX> struct Widen<OpMinMaxF<__nv_bfloat16, Tout, float, MAX>> { using type = OpMinMaxF<float, Tout, float, MAX>; static constexpr bool kWide = true; };
template <class Tout, bool MAX> struct Widen<OpMinMaxF<__half, Tout, float, MAX>> { using type = OpMinMaxF<float, Tout, float, MAX>; static constexpr bool kWide = true; };

// XV consecutive elements at an XV*sizeof(Tin)-aligned shared address, widened to V.
template <class Tin, class V, int XV>
__device__ __forceinline__ void ld_row_vec(const Tin* p, V* out) {
    constexpr int B = XV * (int)sizeof(Tin);
    static_assert(B == 2 || B == 4 || B == 8 || B == 16, "vector width");
    uint32_t w[B >= 4 ? B / 4 : 1];
    if constexpr (B == 16) { const uint4 u = *(const uint4*)p; w[0] = u.x; w[1] = u.y; w[2] = u.z; w[3] = u.w; }
    else if constexpr (B == 8) { const uint2 u = *(const uint2*)p; w[0] = u.x; w[1] = u.y; }
    else if constexpr (B == 4) { w[0] = *(const uint32_t*)p; }
    else { w[0] = *(const uint16_t*)p; }
    if constexpr (std::is_same_v<V, float> && std::is_same_v<Tin, __nv_bfloat16>) {
        // bfloat16 -> float is the 16 bits placed on top of a zero low half
#pragma unroll
        for (int i = 0; i < XV / 2; ++i) {
            out[2 * i] = __uint_as_float(w[i] << 16);
            out[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
        }
    } else if constexpr (std::is_same_v<V, float> && std::is_same_v<Tin, __half>) {
#pragma unroll
        for (int i = 0; i < XV / 2; ++i) {
            __half2 h;
            memcpy(&h, &w[i], 4);
            const float2 f = __half22float2(h);
            out[2 * i] = f.x;
            out[2 * i + 1] = f.y;
        }
    } else {
        static_assert(std::is_same_v<V, Tin>, "only 16-bit floats are widened");
        memcpy(out, w, B);
    }
}

// XV consecutive outputs to global memory: one or two vector stores when `aligned`, else per element
// (with the ragged right edge masked by `nvalid`).
template <class Tout, int XV>
__device__ __forceinline__ void st_row_vec(Tout* d, const Tout* v, bool aligned, int nvalid) {
    constexpr int B = XV * (int)sizeof(Tout);
    if (aligned && nvalid >= XV) {
        if constexpr (B == 32) {
            uint4 u[2];
            memcpy(u, v, 32);
            ((uint4*)d)[0] = u[0];
            ((uint4*)d)[1] = u[1];
        } else if constexpr (B == 16) {
            uint4 u;
            memcpy(&u, v, 16);
            *(uint4*)d = u;
        } else if constexpr (B == 8) {
            uint2 u;
            memcpy(&u, v, 8);
            *(uint2*)d = u;
        } else if constexpr (B == 4) {
            uint32_t u;
            memcpy(&u, v, 4);
            *(uint32_t*)d = u;
        } else {
#pragma unroll
            for (int c = 0; c < XV; ++c) d[c] = v[c];
        }
        return;
    }
#pragma unroll
    for (int c = 0; c < XV; ++c)
        if (c < nvalid) d[c] = v[c];
}

// Register-rotation stream as compute_shape, but each thread owns XV adjacent columns
// (lane*XV .. lane*XV + XV - 1), so one row of its box neighbourhood is NV aligned vector loads
// (the reach PA = R rounded up to XV on each side) instead of one scalar load per tap column, and the
// XV outputs of a row are stored together.  Requires the tile's first column at a shared-memory index
// that is a multiple of XV (the host checks this).  Fold order per output: the table's, as above.
// P: MapParams, or any struct with the same geometry, destination and reduction fields (the batched
// kernel passes a per-tile one).
template <class Tin, class Tout, class Op, class Sh, int XV, int VS, class P>
__device__ __forceinline__ void compute_shape_vec(const P& p, const TileOrigin& o, const Tin* box) {
    using OpV = typename Widen<Op>::type;
    using V = std::conditional_t<Widen<Op>::kWide, float, Tin>;
    constexpr int N = Sh::kN, R = Sh::kR, L = Sh::L;
    constexpr int D = 2 * R + 1;
    constexpr int RY = (N == 3) ? R : 0;
    constexpr int PA = (R + XV - 1) / XV * XV;
    constexpr int NV = 1 + 2 * PA / XV;
    constexpr int NE = NV * XV;
    constexpr int NROW = VS + 2 * R;
    constexpr bool FULL = NROW * L * XV <= 700;
    constexpr auto T = Sh::table;
    static_assert(((N == 3) ? T.o[0].z : T.o[0].y) == -R, "tables start at the lowest stream offset");
    using A = typename OpV::A;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    A acc[D][XV];
    V ctr[D][XV];
#pragma unroll
    for (int q = 0; q < D; ++q)
#pragma unroll
        for (int c = 0; c < XV; ++c) { acc[q][c] = A(0); ctr[q][c] = V(0); }
    const int sr = (N == 3) ? p.bh * p.bw : p.bw;
    const Tin* bb = box + ((N == 3) ? (warp + p.ry - RY) * p.bw : p.rz * p.bh * p.bw + warp * VS * p.bw) +
                    p.padl - PA + lane * XV;
    // the lanes that store outputs (every lane of the warp takes part in the vote)
    const unsigned storing = __ballot_sync(0xffffffffu, (int)min((int64_t)p.tw, p.n[0] - o.x0) - lane * XV > 0);
#ifdef STC_DEBUG_BOUNDS
    {
        // the first and the last element this thread reads lie within the staged box (the whole warp leaves
        // together if one lane fails: the fold below votes across the warp)
        const int64_t n = p.box_bytes / sizeof(Tin), b = bb - box;
        const bool bad = !STC_IN_BOUNDS(b, n, p.status) ||
                         !STC_IN_BOUNDS(b + (NROW - 1) * sr + 2 * RY * p.bw + NE - 1, n, p.status);
        if (__any_sync(0xffffffffu, bad)) return;
    }
#endif
    const int nvx = (int)min((int64_t)p.tw, p.n[0] - o.x0) - lane * XV;   // valid outputs of this thread's XV
    const int nvs = (N == 3) ? (int)min((int64_t)VS, p.n[2] - o.z0) : (int)min((int64_t)VS, p.n[1] - o.y0 - warp * VS);
    const bool row_ok = (N == 3) ? (o.y0 + warp < p.n[1]) : true;
    Tout* dbase = (Tout*)p.dst + p.dst_org + o.x0 + lane * XV +
                  ((N == 3) ? (o.y0 + warp) * p.dstr[1] + o.z0 * p.dstr[2] : (o.y0 + warp * VS) * p.dstr[1]);
    const int64_t dstep = (N == 3) ? p.dstr[2] : p.dstr[1];
    constexpr int VA = (XV * (int)sizeof(Tout)) < 16 ? XV * (int)sizeof(Tout) : 16;
    const bool aligned = (((uintptr_t)((Tout*)p.dst + p.dst_org)) % VA) == 0 &&
                         ((p.dstr[1] * (int64_t)sizeof(Tout)) % VA) == 0 && ((p.dstr[2] * (int64_t)sizeof(Tout)) % VA) == 0;
    auto row = [&](const int r, const int u) {
        V v[2 * RY + 1][NE];
#pragma unroll
        for (int yy = 0; yy < 2 * RY + 1; ++yy)
#pragma unroll
            for (int j = 0; j < NV; ++j) ld_row_vec<Tin, V, XV>(bb + r * sr + yy * p.bw + j * XV, &v[yy][j * XV]);
#pragma unroll
        for (int q = 0; q < D; ++q) {
            const int sidx = r - q;
            if (sidx < 0 || sidx >= VS) continue;
            const int slot = ((u - q) % D + D) % D;
            if (OpV::kZeroInit && q == 0) {
#pragma unroll
                for (int c = 0; c < XV; ++c) acc[slot][c] = OpV::first(V(0), 0);
            }
#pragma unroll
            for (int k = 0; k < L; ++k) {
                const int ko = (N == 3) ? T.o[k].z : T.o[k].y;
                if (ko != q - R) continue;
                const int oy = (N == 3) ? T.o[k].y : 0;
#pragma unroll
                for (int c = 0; c < XV; ++c) {
                    const V val = v[oy + RY][PA + c + T.o[k].x];
                    if (!OpV::kZeroInit && k == 0) acc[slot][c] = OpV::first(val, 0);
                    else acc[slot][c] = OpV::step(acc[slot][c], val, k, p);
                }
            }
            if (OpV::kNeedsCentre && q == R) {
#pragma unroll
                for (int c = 0; c < XV; ++c) ctr[slot][c] = v[RY][PA + c];
            }
            if (q == D - 1 && sidx < nvs && row_ok && nvx > 0) {
                Tout res[XV];
                if constexpr (std::is_same_v<OpV, OpMean<V, Tout, A>> && std::is_same_v<A, float>) {
                    // The Float32 mean's correctly rounded division: when every sum of the warp's row lies
                    // in [2^-90, 3e38] (the range where the FMA-corrected quotient is exact, checked on the
                    // host for this L) all lanes take that quotient after one vote, instead of a range
                    // test and a branch per output; otherwise every output takes the tested division.
                    bool fast = true;
                    float qf[XV];
#pragma unroll
                    for (int c = 0; c < XV; ++c) {
                        fast = fast && fastdiv_in_range(acc[slot][c], p);
                        qf[c] = fastdiv_quotient(acc[slot][c], p);
                    }
                    if (__all_sync(storing, fast)) {
#pragma unroll
                        for (int c = 0; c < XV; ++c) res[c] = from_f32<Tout>(qf[c]);
                    } else {
#pragma unroll
                        for (int c = 0; c < XV; ++c) res[c] = OpV::template finish_c<L>(acc[slot][c], ctr[slot][c], p);
                    }
                } else {
#pragma unroll
                    for (int c = 0; c < XV; ++c) {
                        if constexpr (std::is_same_v<OpV, OpMean<V, Tout, A>>)
                            res[c] = OpV::template finish_c<L>(acc[slot][c], ctr[slot][c], p);
                        else
                            res[c] = OpV::finish(acc[slot][c], ctr[slot][c], p);
                    }
                }
                st_row_vec<Tout, XV>(dbase + sidx * dstep, res, aligned, nvx);
            }
        }
    };
    if constexpr (FULL) {
#pragma unroll
        for (int r = 0; r < NROW; ++r) row(r, r % D);
    } else {
        for (int r0 = 0; r0 < NROW; r0 += D) {
#pragma unroll
            for (int u = 0; u < D; ++u) {
                const int r = r0 + u;
                if (r >= NROW) break;
                row(r, u);
            }
        }
    }
}

// ---------------------------------------------------------------------------- the kernel
// VEC selects compute_shape_vec, with XT then the number of adjacent columns per thread.
template <class Tin, class Tout, class Op, class Sh, int XT, int VS, bool VEC>
__device__ __forceinline__ void map_body(const MapParams& p) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    uint64_t* bars = (uint64_t*)(smem_raw + (size_t)p.stages * p.stage_bytes);
    auto stage_box = [&](int s) { return (Tin*)(smem_raw + (size_t)s * p.stage_bytes); };
    auto compute = [&](const TileOrigin& o, const Tin* box) {
        if constexpr (Sh::kKind == STC_SHAPE_TABLE) compute_generic<Tin, Tout, Op, XT, VS>(p, o, box);
        else if constexpr (VEC) compute_shape_vec<Tin, Tout, Op, Sh, XT, VS>(p, o, box);
        else compute_shape<Tin, Tout, Op, Sh, XT, VS>(p, o, box);
    };
    const int64_t step = gridDim.x;
    if (!p.use_tma) {
        Tin* box = stage_box(0);
        for (int64_t t = blockIdx.x; t < p.ntiles; t += step) {
            const TileOrigin o = tile_origin(p, t);
            load_region<Tin>(p, o, box);
            __syncthreads();
            compute(o, box);
            __syncthreads();
        }
        return;
    }
    const int S = p.stages;
    if (threadIdx.x == 0) {
        prefetch_tensormap(&p.tmap);
        for (int s = 0; s < S; ++s) mbar_init(&bars[s], 1);
        fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0)
        for (int s = 0; s < S - 1; ++s) {
            const int64_t t = blockIdx.x + (int64_t)s * step;
            if (t < p.ntiles) issue_tile_tma(p, tile_origin(p, t), stage_box(s), &bars[s]);
        }
    int it = 0;
    for (int64_t t = blockIdx.x; t < p.ntiles; t += step, ++it) {
        const int s = it % S;
        if (threadIdx.x == 0) {
            const int64_t tn = t + (int64_t)(S - 1) * step;
            if (tn < p.ntiles) {
                fence_proxy_async();
                const int sn = (it + S - 1) % S;
                issue_tile_tma(p, tile_origin(p, tn), stage_box(sn), &bars[sn]);
            }
        }
        const bool ok = mbar_wait_bounded(&bars[s], (uint32_t)((it / S) & 1));
        if (!__syncthreads_and(ok)) {
            // The copy never landed: record it, let in-flight copies drain (bounded), and leave.
            if (threadIdx.x == 0) {
                report(p, DEV_ERR_TIMEOUT);
                for (int k = 0; k < S; ++k) mbar_wait_bounded(&bars[(it + k) % S], (uint32_t)(((it + k) / S) & 1), 100000000ll);
            }
            return;
        }
        const TileOrigin o = tile_origin(p, t);
        Tin* box = stage_box(s);
        if (p.fixup && !region_inside(p, needed_region(p, o))) {
            patch_outside<Tin>(p, o, box);
            fence_proxy_async();
            __syncthreads();
        }
        compute(o, box);
        __syncthreads();
    }
}

template <class Tin, class Tout, class Op, class Sh, int XT, int VS>
__global__ void __launch_bounds__(kMapThreads) map_kernel(const __grid_constant__ MapParams p) {
    map_body<Tin, Tout, Op, Sh, XT, VS, false>(p);
}

// The vector-column variant keeps its XV x (2R+1) accumulators and loaded rows in registers; MINB
// resident CTAs per SM bound its registers (two CTAs: up to 128 per thread).
template <class Tin, class Tout, class Op, class Sh, int XV, int VS, int MINB>
__global__ void __launch_bounds__(kMapThreads, MINB) map_vec_kernel(const __grid_constant__ MapParams p) {
    map_body<Tin, Tout, Op, Sh, XV, VS, true>(p);
}

}  // namespace stc
