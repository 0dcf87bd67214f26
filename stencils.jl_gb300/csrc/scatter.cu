// scatter.cu — scatterstencil!(f, op, dest, source) as a deterministic gather.
//
// Replaces scatterstencil! (src/scatterstencil.jl:36-133).  The reference pushes each source cell's
// values to its neighbours in passes over columns 2R + 1 apart, so no two threads of a pass write the
// same cell.  Here one thread owns each dest cell and pulls every contribution that lands on it, in the
// order the reference's pass schedule delivers them when run on one thread: (pass of the source
// column, source column, source row, offset).  No atomics, and the result is bit-exact with that order
// for every combine op, including floating-point +.
#include <algorithm>
#include <tuple>
#include <vector>

#include "common.cuh"
#include "dispatch.h"
#include "profile.h"

namespace stc {

constexpr int kScatterMaxLen = 256;
constexpr int kScatterPermMax = 2048;   // (2R + 1) * L entries of the interior orders

struct ScatterParams {
    const void* src;
    void* dst;
    int64_t sst1, sorg;        // source parent row stride and offset of logical (0, 0)
    int64_t dst1;              // dest row stride
    int64_t ny, nx;            // logical size (axis 0, axis 1)
    int32_t L, R, boundary, value, combine;
    double constant;
    int32_t perm_ok;           // interior cells use perm (else every cell runs the selection loop)
    int8_t off[kScatterMaxLen][2];
    double w[kScatterMaxLen];
    // For a dest cell far enough from every edge (R, or R + 1 under Reflect) each offset k brings
    // exactly one contribution, from
    // (ti - o0, tj - o1); their order depends only on tj mod (2R + 1): perm[(tj mod (2R+1)) * L + i]
    // is the i-th offset in (pass, source row, offset) order.
    uint8_t perm[kScatterPermMax];
};

// Source coordinates u on one axis whose target u + o maps to t (at most 3): Remove/Use only u + o = t;
// Wrap u + o = t (mod n); Reflect u + o = t, -t or 2n - 2 - t (src/scatterstencil.jl:76-112).
__device__ __forceinline__ int scatter_sources(int boundary, int64_t t, int64_t o, int64_t n, int64_t* s) {
    int c = 0;
    auto add = [&](int64_t u) {
        const int64_t v = u - o;
        if (v >= 0 && v < n) s[c++] = v;
    };
    if (boundary == STC_WRAP) {
        add(t);
        add(t - n);
        add(t + n);
    } else if (boundary == STC_REFLECT) {
        add(t);
        if (t >= 1) add(-t);
        if (t <= n - 2) add(2 * n - 2 - t);
    } else {
        add(t);
    }
    return c;
}

template <class T> __device__ __forceinline__ T sc_add(T a, T b);
template <> __device__ __forceinline__ double sc_add<double>(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float sc_add<float>(float a, float b) { return __fadd_rn(a, b); }
template <class T> __device__ __forceinline__ T sc_mul(T a, T b);
template <> __device__ __forceinline__ double sc_mul<double>(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float sc_mul<float>(float a, float b) { return __fmul_rn(a, b); }

template <class T>
__global__ void __launch_bounds__(256) scatter_kernel(const __grid_constant__ ScatterParams p) {
    const T* src = (const T*)p.src;
    T* dst = (T*)p.dst;
    const int64_t total = p.ny * p.nx;
    const int64_t stride = 2 * (int64_t)p.R + 1;
    for (int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lin < total;
         lin += (int64_t)gridDim.x * blockDim.x) {
        const int64_t ti = lin % p.ny, tj = lin / p.ny;
        T acc = dst[ti + tj * p.dst1];
        auto combine = [&](T val) {
            if (p.combine == STC_COMBINE_ADD) acc = sc_add<T>(acc, val);
            else if (p.combine == STC_COMBINE_MAX) acc = jl_max(acc, val);
            else acc = jl_min(acc, val);
        };
        auto value = [&](int k, int64_t si, int64_t sj) -> T {
            if (p.value == STC_SCATTER_CONST) return (T)p.constant;
            const T c = src[p.sorg + si + sj * p.sst1];
            return p.value == STC_SCATTER_CENTER ? c : sc_mul<T>(c, (T)p.w[k]);
        };
        // interior: no source's target is wrapped or reflected onto this cell (Reflect maps the edge
        // row's x - R onto x + R, so it needs one more cell of margin)
        const int m = p.R + (p.boundary == STC_REFLECT ? 1 : 0);
        if (p.perm_ok && ti >= m && ti < p.ny - m && tj >= m && tj < p.nx - m) {
            const uint8_t* order = p.perm + (tj % stride) * p.L;
            for (int i = 0; i < p.L; ++i) {
                const int k = order[i];
                combine(value(k, ti - p.off[k][0], tj - p.off[k][1]));
            }
            dst[ti + tj * p.dst1] = acc;
            continue;
        }
        // Visit contributions in increasing (pass, column, row, offset): each round picks the smallest
        // key above the previous one among all candidates (a handful per cell).
        int64_t pk = -1, pj = -1, pi = -1, pkk = -1;
        while (true) {
            int64_t bk = INT64_MAX, bj = 0, bi = 0, bkk = 0;
            for (int k = 0; k < p.L; ++k) {
                int64_t si[3], sj[3];
                const int ni = scatter_sources(p.boundary, ti, p.off[k][0], p.ny, si);
                const int nj = scatter_sources(p.boundary, tj, p.off[k][1], p.nx, sj);
                for (int a = 0; a < ni; ++a)
                    for (int b = 0; b < nj; ++b) {
                        const int64_t pas = sj[b] % stride;
                        // lexicographic (pass, column, row, offset) > previous and < best
                        auto gt = [&](int64_t x0, int64_t x1, int64_t x2, int64_t x3, int64_t y0, int64_t y1, int64_t y2,
                                      int64_t y3) {
                            if (x0 != y0) return x0 > y0;
                            if (x1 != y1) return x1 > y1;
                            if (x2 != y2) return x2 > y2;
                            return x3 > y3;
                        };
                        if (!gt(pas, sj[b], si[a], k, pk, pj, pi, pkk)) continue;
                        if (bk != INT64_MAX && !gt(bk, bj, bi, bkk, pas, sj[b], si[a], k)) continue;
                        bk = pas; bj = sj[b]; bi = si[a]; bkk = k;
                    }
            }
            if (bk == INT64_MAX) break;
            combine(value((int)bkk, bi, bj));
            pk = bk; pj = bj; pi = bi; pkk = bkk;
        }
        dst[ti + tj * p.dst1] = acc;
    }
}

}  // namespace stc

using namespace stc;

extern "C" {

int stc_scatter(const stc_grid* src, const stc_grid* dst, const stc_stencil* st, const stc_scatter_op* op,
                const stc_bc* bc, void* stream, uint32_t flags) {
    if (!src || !dst || !st || !op || !bc || !src->data || !dst->data || !st->offsets) return STC_ERR_INVALID;
    if (src->ndims != 2 || dst->ndims != 2 || st->ndims != 2) return STC_ERR_UNSUPPORTED;
    if (src->dtype != dst->dtype || (src->dtype != STC_F64 && src->dtype != STC_F32)) return STC_ERR_UNSUPPORTED;
    if (neighbor_dtype(src->dtype, bc) != src->dtype) return STC_ERR_UNSUPPORTED;   // padval promotion
    if ((src->size[0] > 1 && src->stride[0] != 1) || (dst->size[0] > 1 && dst->stride[0] != 1)) return STC_ERR_INVALID;
    if (op->value < STC_SCATTER_CONST || op->value > STC_SCATTER_WEIGHTED) return STC_ERR_UNSUPPORTED;
    if (op->combine < STC_COMBINE_ADD || op->combine > STC_COMBINE_MIN) return STC_ERR_UNSUPPORTED;
    if (op->value == STC_SCATTER_WEIGHTED && !st->weights) return STC_ERR_KERNEL_LENGTH;
    if (st->len < 1 || st->len > kScatterMaxLen || st->radius < 0 || st->radius > STC_MAX_RADIUS)
        return STC_ERR_UNSUPPORTED;
    const int R = st->radius;
    for (int d = 0; d < 2; ++d)
        if (!(R < src->size[d])) return STC_ERR_RADIUS;
    const bool halo = bc->padding != STC_CONDITIONAL;
    if (bc->boundary == STC_USE && !halo) return STC_ERR_UNSUPPORTED;   // no getneighbor method for it
    static thread_local ScatterParams p;
    memset(&p, 0, sizeof(p));
    p.ny = src->size[0] - (halo ? 2 * R : 0);
    p.nx = src->size[1] - (halo ? 2 * R : 0);
    if (p.ny < 0 || p.nx < 0) return STC_ERR_RADIUS;
    if (dst->size[0] != p.ny || dst->size[1] != p.nx) return STC_ERR_SIZE_MISMATCH;
    for (int d = 0; d < 2; ++d)
        if (src->stride[d] < 0 || dst->stride[d] < 0) return STC_ERR_INVALID;
    if (grids_overlap(src, dst)) return STC_ERR_INVALID;   // a dest cell's pull would read cells being written
    p.src = src->data;
    p.dst = dst->data;
    p.sst1 = src->stride[1];
    p.sorg = halo ? (int64_t)R * (1 + src->stride[1]) : 0;
    p.dst1 = dst->stride[1];
    p.L = st->len;
    p.R = R;
    p.boundary = bc->boundary;
    p.value = op->value;
    p.combine = op->combine;
    const bool f32 = src->dtype == STC_F32;
    p.constant = f32 ? (double)(float)op->constant : op->constant;
    for (int k = 0; k < st->len; ++k) {
        const int ox = st->offsets[2 * k], oy = st->offsets[2 * k + 1];
        if (ox > R || ox < -R || oy > R || oy < -R) return STC_ERR_UNSUPPORTED;
        p.off[k][0] = (int8_t)ox;
        p.off[k][1] = (int8_t)oy;
        if (st->weights) p.w[k] = f32 ? (double)(float)st->weights[k] : st->weights[k];
    }
    // interior orders: sort the offsets by (pass of the source column, source row, offset) for each
    // residue of the dest column; offsets are distinct, so the pass separates different columns
    const int stride = 2 * R + 1;
    p.perm_ok = stride * st->len <= kScatterPermMax && st->len <= 256;
    if (p.perm_ok)
        for (int r = 0; r < stride; ++r) {
            std::vector<int> ks(st->len);
            for (int k = 0; k < st->len; ++k) ks[k] = k;
            auto key = [&](int k) {
                const int o0 = st->offsets[2 * k], o1 = st->offsets[2 * k + 1];
                const int pass = ((r - o1) % stride + stride) % stride;
                return std::make_tuple(pass, -o0, k);   // source row ti - o0 ascending
            };
            std::sort(ks.begin(), ks.end(), [&](int x, int y) { return key(x) < key(y); });
            for (int i = 0; i < st->len; ++i) p.perm[r * st->len + i] = (uint8_t)ks[i];
        }
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    if ((rc = launch_halo_fill(src, R, bc, s))) return rc;   // update_boundary!(source)
    const int64_t total = p.ny * p.nx;
    if (total > 0) {
        const int64_t blocks = std::min<int64_t>((total + 255) / 256, (int64_t)ctx->num_sms * 16);
        void* prof = prof_begin(s);
        if (f32) scatter_kernel<float><<<(unsigned)blocks, 256, 0, s>>>(p);
        else scatter_kernel<double><<<(unsigned)blocks, 256, 0, s>>>(p);
        prof_end(prof, s, "scatter", (double)total * 3 * dtype_size(src->dtype), (double)total);
        if ((rc = cuda_fail(cudaGetLastError()))) return rc;
    }
    if (!(flags & STC_ASYNC)) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e);
    }
    return STC_OK;
}

}  // extern "C"
