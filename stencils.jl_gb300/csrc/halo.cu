// halo.cu — K2, update_boundary!: write the halo ring of a Halo-padded parent from its interior.
//
// Replaces the @generated update_boundary! (src/array.jl:202-233) and halo_val (:235-239).  For
// each axis i the two slabs of width R along i span the full padded extent of the other axes;
// a cell gets padval (Remove) or the interior value at bounded_index of its coordinates
// (Wrap / Reflect, src/array.jl:154-179).  Every halo cell depends only on interior cells, so the
// slabs are written in one launch; cells shared by two slabs receive the same value from both.
#include "common.cuh"
#include "dispatch.h"
#include "profile.h"

namespace stc {

struct HaloParams {
    void* base;
    int64_t st[3];
    int64_t n[3];        // logical size
    int64_t slab_cells[6];
    int64_t total;
    int32_t R, ndims, boundary;
    double padf;
    int64_t padi;
};

__device__ __forceinline__ int64_t hb(int boundary, int64_t i, int64_t s) {
    if (boundary == STC_WRAP) return i < 0 ? i + s : (i >= s ? i - s : i);
    return i < 0 ? -i : (i >= s ? 2 * s - 2 - i : i);
}

template <class T> __device__ __forceinline__ T halo_pad(const HaloParams& p);
template <> __device__ __forceinline__ double halo_pad<double>(const HaloParams& p) { return p.padf; }
template <> __device__ __forceinline__ float halo_pad<float>(const HaloParams& p) { return (float)p.padf; }
template <> __device__ __forceinline__ __nv_bfloat16 halo_pad<__nv_bfloat16>(const HaloParams& p) {
    return __float2bfloat16_rn((float)p.padf);
}
template <> __device__ __forceinline__ __half halo_pad<__half>(const HaloParams& p) { return __double2half(p.padf); }
template <> __device__ __forceinline__ uint8_t halo_pad<uint8_t>(const HaloParams& p) { return (uint8_t)p.padi; }
template <> __device__ __forceinline__ int32_t halo_pad<int32_t>(const HaloParams& p) {
    return (int32_t)(uint32_t)(uint64_t)p.padi;
}
template <> __device__ __forceinline__ int64_t halo_pad<int64_t>(const HaloParams& p) { return p.padi; }

template <class T>
__global__ void halo_fill_kernel(const HaloParams p) {
    T* base = (T*)p.base;
    const int64_t R = p.R;
    for (int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lin < p.total;
         lin += (int64_t)gridDim.x * blockDim.x) {
        // locate the slab
        int slab = 0;
        int64_t r = lin;
        while (slab < 2 * p.ndims - 1 && r >= p.slab_cells[slab]) r -= p.slab_cells[slab++];
        const int ax = slab >> 1, side = slab & 1;
        int64_t ext[3], J[3];
        for (int d = 0; d < 3; ++d) ext[d] = d < p.ndims ? (d == ax ? R : p.n[d] + 2 * R) : 1;
        J[0] = r % ext[0];
        J[1] = (r / ext[0]) % ext[1];
        J[2] = r / (ext[0] * ext[1]);
        // to logical coordinates
        for (int d = 0; d < p.ndims; ++d) {
            if (d == ax) J[d] = side == 0 ? J[d] - R : p.n[d] + J[d];
            else J[d] -= R;
        }
        const int64_t dsto = (J[0] + R) + (p.ndims > 1 ? (J[1] + R) * p.st[1] : 0) +
                             (p.ndims > 2 ? (J[2] + R) * p.st[2] : 0);
        T v;
        if (p.boundary == STC_REMOVE) {
            v = halo_pad<T>(p);
        } else {
            int64_t B[3] = {0, 0, 0};
            for (int d = 0; d < p.ndims; ++d) B[d] = hb(p.boundary, J[d], p.n[d]);
            v = base[(B[0] + R) + (p.ndims > 1 ? (B[1] + R) * p.st[1] : 0) + (p.ndims > 2 ? (B[2] + R) * p.st[2] : 0)];
        }
        base[dsto] = v;
    }
}

int launch_halo_fill(const stc_grid* g, int radius, const stc_bc* bc, cudaStream_t stream) {
    if (bc->padding == STC_CONDITIONAL || bc->boundary == STC_USE || radius == 0) return STC_OK;
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    HaloParams p{};
    p.base = g->data;
    p.R = radius;
    p.ndims = g->ndims;
    p.boundary = bc->boundary;
    p.padf = bc->padval;
    p.padi = bc->padval_int;
    for (int d = 0; d < 3; ++d) {
        p.st[d] = d < g->ndims ? g->stride[d] : 0;
        p.n[d] = d < g->ndims ? g->size[d] - 2 * radius : 1;
    }
    for (int d = 0; d < g->ndims; ++d)
        if (p.n[d] < 1) return STC_OK;  // nothing inside to copy from; the reference has no cells to map
    p.total = 0;
    for (int s = 0; s < 2 * g->ndims; ++s) {
        const int ax = s >> 1;
        int64_t c = 1;
        for (int d = 0; d < g->ndims; ++d) c *= (d == ax) ? radius : p.n[d] + 2 * radius;
        p.slab_cells[s] = c;
        p.total += c;
    }
    const int threads = 256;
    int64_t blocks = (p.total + threads - 1) / threads;
    if (blocks > (int64_t)ctx->num_sms * 8) blocks = (int64_t)ctx->num_sms * 8;
    if (blocks < 1) blocks = 1;
    void* prof = prof_begin(stream);
    switch (g->dtype) {
    case STC_F64: halo_fill_kernel<double><<<(int)blocks, threads, 0, stream>>>(p); break;
    case STC_F32: halo_fill_kernel<float><<<(int)blocks, threads, 0, stream>>>(p); break;
    case STC_BF16: halo_fill_kernel<__nv_bfloat16><<<(int)blocks, threads, 0, stream>>>(p); break;
    case STC_F16: halo_fill_kernel<__half><<<(int)blocks, threads, 0, stream>>>(p); break;
    case STC_U8: case STC_BOOL: halo_fill_kernel<uint8_t><<<(int)blocks, threads, 0, stream>>>(p); break;
    case STC_I32: halo_fill_kernel<int32_t><<<(int)blocks, threads, 0, stream>>>(p); break;
    case STC_I64: halo_fill_kernel<int64_t><<<(int)blocks, threads, 0, stream>>>(p); break;
    default: return STC_ERR_UNSUPPORTED;
    }
    prof_end(prof, stream, "halo_fill", (double)p.total * 2 * dtype_size(g->dtype), (double)p.total);
    return cuda_fail(cudaGetLastError());
}

}  // namespace stc
