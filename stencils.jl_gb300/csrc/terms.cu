// terms.cu — maps over several arrays: dest[I] = t_1 + t_2 + ... with one term per argument.
//
// Replaces gatherstencil!(f, dest, source, args...) (src/gatherstencil.jl:84-113) for the registered
// f that sums per-argument terms: center(hood), sum / mean / kernelproduct of the neighbours, or the
// value of a plain array at I (`_getarg`, src/gatherstencil.jl:111-112), each optionally scaled.
// One thread per output cell gathers every term straight from global memory (L1/L2 cached; the
// arguments' stencils and boundaries differ, so there is no shared tile); every operation is an
// explicit round-to-nearest one, in the grids' element type, in the reference's left-to-right order.
#include <algorithm>

#include "common.cuh"
#include "dispatch.h"
#include "profile.h"

namespace stc {

struct TermDev {
    const void* src;
    int64_t st[3];          // parent strides (0 beyond ndims)
    int64_t org;            // parent offset of logical (0, 0, 0)
    int64_t n[3];           // logical size (1 beyond ndims)
    int32_t kind, scaled, L, halo, boundary, nd;
    double alpha, padf;
    int8_t off[STC_MAX_TERM_LEN][3];
    double w[STC_MAX_TERM_LEN];
};

struct TermsParams {
    TermDev t[STC_MAX_TERMS];
    int32_t nterms, nd;
    void* dst;
    int64_t dstr[3];
    int64_t dst_org;
    int64_t n[3];
};

template <class T> __device__ __forceinline__ T t_add(T a, T b);
template <> __device__ __forceinline__ double t_add<double>(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ float t_add<float>(float a, float b) { return __fadd_rn(a, b); }
template <class T> __device__ __forceinline__ T t_mul(T a, T b);
template <> __device__ __forceinline__ double t_mul<double>(double a, double b) { return __dmul_rn(a, b); }
template <> __device__ __forceinline__ float t_mul<float>(float a, float b) { return __fmul_rn(a, b); }
template <class T> __device__ __forceinline__ T t_div(T a, T b);
template <> __device__ __forceinline__ double t_div<double>(double a, double b) { return __ddiv_rn(a, b); }
template <> __device__ __forceinline__ float t_div<float>(float a, float b) { return __fdiv_rn(a, b); }

__device__ __forceinline__ int64_t t_bound(int boundary, int64_t i, int64_t s) {
    if (boundary == STC_WRAP) return i < 0 ? i + s : (i >= s ? i - s : i);
    return i < 0 ? -i : (i >= s ? 2 * s - 2 - i : i);
}

// Neighbour k of argument t at logical I: Halo reads the parent (ring included); Conditional applies
// Remove / Wrap / Reflect outside the array (src/array.jl:129-188).
template <class T>
__device__ __forceinline__ T t_neighbour(const TermDev& t, int64_t x, int64_t y, int64_t z, int k) {
    const T* s = (const T*)t.src;
    x += t.off[k][0];
    y += t.off[k][1];
    z += t.off[k][2];
    if (!t.halo && (x < 0 || x >= t.n[0] || y < 0 || y >= t.n[1] || z < 0 || z >= t.n[2])) {
        if (t.boundary == STC_REMOVE) return (T)t.padf;
        x = t_bound(t.boundary, x, t.n[0]);
        if (t.nd > 1) y = t_bound(t.boundary, y, t.n[1]);
        if (t.nd > 2) z = t_bound(t.boundary, z, t.n[2]);
    }
    return s[t.org + x + y * t.st[1] + z * t.st[2]];
}

template <class T>
__device__ __forceinline__ T t_term(const TermDev& t, int64_t x, int64_t y, int64_t z) {
    const T* s = (const T*)t.src;
    T g;
    switch (t.kind) {
    case STC_TERM_CENTER:
    case STC_TERM_VALUE:
        g = s[t.org + x + y * t.st[1] + z * t.st[2]];
        break;
    case STC_TERM_KDOT: {
        // kernelproduct: s = zero(T); s += hood[k] * kernel[k], product and sum rounded separately
        g = T(0);
        for (int k = 0; k < t.L; ++k) g = t_add<T>(g, t_mul<T>(t_neighbour<T>(t, x, y, z, k), (T)t.w[k]));
        break;
    }
    default: {
        // sum / mean of the neighbours: first element as is, then + in offset order
        g = t_neighbour<T>(t, x, y, z, 0);
        for (int k = 1; k < t.L; ++k) g = t_add<T>(g, t_neighbour<T>(t, x, y, z, k));
        if (t.kind == STC_TERM_MEAN) g = t_div<T>(g, (T)t.L);
        break;
    }
    }
    return t.scaled ? t_mul<T>((T)t.alpha, g) : g;
}

template <class T>
__global__ void __launch_bounds__(256) terms_kernel(const __grid_constant__ TermsParams p) {
    const int64_t total = p.n[0] * p.n[1] * p.n[2];
    T* dst = (T*)p.dst;
    for (int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lin < total;
         lin += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = lin % p.n[0], r = lin / p.n[0];
        const int64_t y = r % p.n[1], z = r / p.n[1];
        T acc = t_term<T>(p.t[0], x, y, z);
        for (int m = 1; m < p.nterms; ++m) acc = t_add<T>(acc, t_term<T>(p.t[m], x, y, z));
        dst[p.dst_org + x + y * p.dstr[1] + z * p.dstr[2]] = acc;
    }
}

}  // namespace stc

using namespace stc;

extern "C" {

int stc_map_terms(const stc_term* terms, int32_t nterms, const stc_grid* dst, int32_t dst_padded, void* stream,
                  uint32_t flags) {
    if (!terms || !dst || nterms < 1 || nterms > STC_MAX_TERMS || !dst->data) return STC_ERR_INVALID;
    const int dt = dst->dtype;
    if (dt != STC_F64 && dt != STC_F32) return STC_ERR_UNSUPPORTED;
    static thread_local TermsParams p;
    memset(&p, 0, sizeof(p));
    int64_t n[3] = {1, 1, 1};
    const int nd = dst->ndims;
    if (nd < 1 || nd > 3 || (dst->size[0] > 1 && dst->stride[0] != 1)) return STC_ERR_INVALID;
    for (int d = 0; d < nd; ++d)
        if (dst->size[d] < 0 || dst->stride[d] < 0) return STC_ERR_INVALID;
    for (int m = 0; m < nterms; ++m) {
        const stc_term& tm = terms[m];
        const stc_grid* g = tm.grid;
        if (!g || !g->data || g->ndims != nd || (g->size[0] > 1 && g->stride[0] != 1)) return STC_ERR_INVALID;
        for (int d = 0; d < nd; ++d)
            if (g->size[d] < 0 || g->stride[d] < 0) return STC_ERR_INVALID;
        if (g->dtype != dt) return STC_ERR_UNSUPPORTED;
        if (tm.bc && neighbor_dtype(g->dtype, tm.bc) != g->dtype) return STC_ERR_UNSUPPORTED;   // padval promotion
        if (grids_overlap(g, dst)) return STC_ERR_INVALID;   // dest may not share memory with an argument
        if (tm.kind < STC_TERM_CENTER || tm.kind > STC_TERM_VALUE) return STC_ERR_UNSUPPORTED;
        TermDev& t = p.t[m];
        t.src = g->data;
        t.kind = tm.kind;
        t.scaled = tm.scaled != 0;
        t.alpha = tm.alpha;
        t.nd = nd;
        int R = 0;
        if (tm.kind == STC_TERM_VALUE) {
            t.halo = 0;
        } else {
            const stc_stencil* st = tm.stencil;
            const stc_bc* bc = tm.bc;
            if (!st || !bc || !st->offsets) return STC_ERR_INVALID;
            if (st->ndims < 1 || st->ndims > nd || st->len < 1) return STC_ERR_INVALID;
            if (st->len > STC_MAX_TERM_LEN || st->radius > STC_MAX_RADIUS) return STC_ERR_UNSUPPORTED;
            if (tm.kind == STC_TERM_KDOT && !st->weights) return STC_ERR_KERNEL_LENGTH;
            if (tm.kind == STC_TERM_KDOT && dt == STC_F32 && st->weight_dtype != STC_F32) return STC_ERR_UNSUPPORTED;
            if (bc->boundary == STC_USE && bc->padding == STC_CONDITIONAL) return STC_ERR_UNSUPPORTED;
            R = st->radius;
            for (int d = 0; d < nd; ++d)
                if (!(R < g->size[d])) return STC_ERR_RADIUS;
            for (int k = 0; k < st->len; ++k)
                for (int d = 0; d < 3; ++d) {
                    const int o = d < st->ndims ? st->offsets[k * st->ndims + d] : 0;
                    if (o > R || o < -R) return STC_ERR_UNSUPPORTED;
                    t.off[k][d] = (int8_t)o;
                }
            if (st->weights)
                for (int k = 0; k < st->len; ++k)
                    t.w[k] = dt == STC_F32 ? (double)(float)st->weights[k] : st->weights[k];
            t.L = st->len;
            t.halo = bc->padding != STC_CONDITIONAL;
            t.boundary = bc->boundary;
            t.padf = dt == STC_F32 ? (double)(float)bc->padval : bc->padval;
            if (!t.halo) R = 0;
        }
        for (int d = 0; d < 3; ++d) {
            t.n[d] = d < nd ? g->size[d] - 2 * R : 1;
            t.st[d] = d < nd ? g->stride[d] : 0;
            t.org += (int64_t)R * t.st[d];
            if (t.n[d] < 0) return STC_ERR_RADIUS;
        }
        // every argument has the first one's logical size (src/gatherstencil.jl:118-124)
        for (int d = 0; d < 3; ++d) {
            if (m == 0) n[d] = t.n[d];
            else if (t.n[d] != n[d]) return STC_ERR_SIZE_MISMATCH;
        }
    }
    // dest: the logical size, or (dst_padded) the first argument's padded parent size
    const int R0 = (terms[0].kind != STC_TERM_VALUE && terms[0].bc->padding != STC_CONDITIONAL)
                       ? terms[0].stencil->radius : 0;
    for (int d = 0; d < nd; ++d) {
        const int64_t want = n[d] + (dst_padded ? 2 * R0 : 0);
        if (dst->size[d] != want) return STC_ERR_SIZE_MISMATCH;
        p.dstr[d] = dst->stride[d];
        if (dst_padded) p.dst_org += (int64_t)R0 * dst->stride[d];
    }
    for (int d = 0; d < 3; ++d) p.n[d] = n[d];
    p.nterms = nterms;
    p.nd = nd;
    p.dst = dst->data;
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    cudaStream_t s = (cudaStream_t)stream;
    // update_boundary! on every Halo argument first (src/gatherstencil.jl:92-94)
    for (int m = 0; m < nterms; ++m)
        if (terms[m].kind != STC_TERM_VALUE && (rc = launch_halo_fill(terms[m].grid, terms[m].stencil->radius,
                                                                       terms[m].bc, s)))
            return rc;
    const int64_t total = n[0] * n[1] * n[2];
    if (total > 0) {
        const int64_t blocks = std::min<int64_t>((total + 255) / 256, (int64_t)ctx->num_sms * 16);
        void* prof = prof_begin(s);
        if (dt == STC_F64) terms_kernel<double><<<(unsigned)blocks, 256, 0, s>>>(p);
        else terms_kernel<float><<<(unsigned)blocks, 256, 0, s>>>(p);
        const int es = dtype_size(dt);
        prof_end(prof, s, "terms", (double)total * es * (nterms + 1), (double)total);
        if ((rc = cuda_fail(cudaGetLastError()))) return rc;
    }
    if (!(flags & STC_ASYNC)) {
        cudaError_t e = cudaStreamSynchronize(s);
        if (e != cudaSuccess) return cuda_fail(e);
    }
    return STC_OK;
}

}  // extern "C"
