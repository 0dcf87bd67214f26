// halo.cu — K2, update_boundary!: write the halo ring of a Halo-padded parent from its interior.
//
// Replaces the @generated update_boundary! (src/array.jl:202-233) and halo_val (:235-239).  For
// each axis i the two slabs of width R along i span the full padded extent of the other axes;
// a cell gets padval (Remove) or the interior value at bounded_index of its coordinates
// (Wrap / Reflect, src/array.jl:154-179).  Every halo cell depends only on interior cells, so the
// slabs are written in one launch; cells shared by two slabs receive the same value from both.
#include <algorithm>
#include <cstdint>
#include <type_traits>

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

// Every ring cell exactly once, in three parts (e = ring width on an axis, 0 beyond ndims):
//   A  the z-ring planes, whole (rows y in [-e1, n1+e1), x along the threads);
//   B  the y-ring rows of the interior planes (x along the threads);
//   C  the x-ring cells of the interior rows (one cell per thread).
// A ring cell holds padval (Remove) or the interior cell at bounded_index of its coordinates on every
// axis (Wrap / Reflect).  Rows are indexed in 32-bit (axes < 2^31), so no per-cell 64-bit division.
template <class T>
__device__ __forceinline__ T halo_value(const HaloParams& p, const T* base, int64_t x, int64_t y, int64_t z) {
    if (p.boundary == STC_REMOVE) return halo_pad<T>(p);
    const int64_t bx = hb(p.boundary, x, p.n[0]);
    const int64_t by = p.ndims > 1 ? hb(p.boundary, y, p.n[1]) : 0;
    const int64_t bz = p.ndims > 2 ? hb(p.boundary, z, p.n[2]) : 0;
    return base[(bx + p.R) + (p.ndims > 1 ? (by + p.R) * p.st[1] : 0) + (p.ndims > 2 ? (bz + p.R) * p.st[2] : 0)];
}

template <class T>
__global__ void halo_fill_kernel(const HaloParams p) {
    T* base = (T*)p.base;
    const int e0 = p.R, e1 = p.ndims > 1 ? p.R : 0, e2 = p.ndims > 2 ? p.R : 0;
    const int n0 = (int)p.n[0], n1 = (int)p.n[1], n2 = (int)p.n[2];
    const int wx = n0 + 2 * e0, wy = n1 + 2 * e1;
    const int64_t rowsA = (int64_t)2 * e2 * wy, rowsB = (int64_t)n2 * 2 * e1;
    const int64_t cellsC = (int64_t)n1 * n2 * 2 * e0;
    auto put = [&](int64_t x, int64_t y, int64_t z) {
        base[(x + p.R) + (y + e1) * p.st[1] + (z + e2) * p.st[2]] = halo_value<T>(p, base, x, y, z);
    };
    // parts A and B: a block per row, threads along x
    for (int64_t r = blockIdx.x; r < rowsA + rowsB; r += gridDim.x) {
        int64_t y, z;
        if (r < rowsA) {
            const int zi = (int)(r / wy);   // < 2 e2
            y = r - (int64_t)zi * wy - e1;
            z = zi < e2 ? zi - e2 : n2 + (zi - e2);
        } else {
            const int64_t q = r - rowsA;
            const int64_t zi = q / (2 * e1), yi = q - zi * 2 * e1;
            z = zi;
            y = yi < e1 ? yi - e1 : n1 + (yi - e1);
        }
        for (int xi = threadIdx.x; xi < wx; xi += blockDim.x) put(xi - e0, y, z);
    }
    // part C: one x-ring cell per thread (32-bit indices while they fit)
    if (cellsC < (1ll << 31)) {
        const int cc = (int)cellsC, w = 2 * e0;
        for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < cc; c += gridDim.x * blockDim.x) {
            const int row = c / w, j = c - row * w;
            const int z = row / n1, y = row - z * n1;
            put(j < e0 ? j - e0 : n0 + (j - e0), y, z);
        }
        return;
    }
    for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < cellsC; c += (int64_t)gridDim.x * blockDim.x) {
        const int64_t row = c / (2 * e0);
        const int j = (int)(c - row * 2 * e0);
        const int64_t y = row % n1, z = row / n1;
        put(j < e0 ? j - e0 : n0 + (j - e0), y, z);
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
    for (int d = 0; d < 3; ++d)
        if (p.n[d] + 2 * radius >= (1ll << 31)) return STC_ERR_UNSUPPORTED;
    const int threads = 256;
    int64_t blocks = (p.total + threads - 1) / threads;
    if (blocks > (int64_t)ctx->num_sms * 6) blocks = (int64_t)ctx->num_sms * 6;   // one wave (6 CTAs/SM resident)
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

// ------------------------------------------------------------------ box copy between parents
// dst[dorg + x + y*ds1 + z*ds2] = src[sorg + x + y*ss1 + z*ss2] over an n0 x n1 x n2 box: a block per
// row (y, z), threads along x, so no per-element division.
struct CopyParams {
    const void* src;
    void* dst;
    int64_t sorg, ss1, ss2, dorg, ds1, ds2;
    int64_t n0, n1, rows;
};

template <class T>
__global__ void grid_copy_kernel(const CopyParams p) {
    const T* src = (const T*)p.src;
    T* dst = (T*)p.dst;
    for (int64_t row = blockIdx.x; row < p.rows; row += gridDim.x) {
        const int64_t y = row % p.n1, z = row / p.n1;
        const T* s = src + p.sorg + y * p.ss1 + z * p.ss2;
        T* d = dst + p.dorg + y * p.ds1 + z * p.ds2;
        for (int64_t x = threadIdx.x; x < p.n0; x += blockDim.x) d[x] = s[x];
    }
}

int launch_grid_copy(const stc_grid* src, int64_t sorg, const stc_grid* dst, int64_t dorg, const int64_t n[3],
                     cudaStream_t stream) {
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    CopyParams p{};
    p.src = src->data;
    p.dst = dst->data;
    p.sorg = sorg;
    p.dorg = dorg;
    p.ss1 = src->ndims > 1 ? src->stride[1] : 0;
    p.ss2 = src->ndims > 2 ? src->stride[2] : 0;
    p.ds1 = dst->ndims > 1 ? dst->stride[1] : 0;
    p.ds2 = dst->ndims > 2 ? dst->stride[2] : 0;
    p.n0 = n[0];
    p.n1 = n[1];
    p.rows = n[1] * n[2];
    if (p.n0 < 1 || p.rows < 1) return STC_OK;
    const int threads = p.n0 >= 256 ? 256 : 128;
    const int blocks = (int)std::min<int64_t>(p.rows, (int64_t)ctx->num_sms * 16);
    switch (dtype_size(src->dtype)) {
    case 8: grid_copy_kernel<uint64_t><<<blocks, threads, 0, stream>>>(p); break;
    case 4: grid_copy_kernel<uint32_t><<<blocks, threads, 0, stream>>>(p); break;
    case 2: grid_copy_kernel<uint16_t><<<blocks, threads, 0, stream>>>(p); break;
    case 1: grid_copy_kernel<uint8_t><<<blocks, threads, 0, stream>>>(p); break;
    default: return STC_ERR_UNSUPPORTED;
    }
    return cuda_fail(cudaGetLastError());
}

// ------------------------------------------------------------------ box conversion between element types
// Julia's convert(TO, x): into a float type round to nearest; into an integer type only an exactly
// representable value (else InexactError: the status bit), into Bool only 0 or 1.  Integer sources go
// through Float64 into a 16-bit float (exact below 2^53).
template <class TI> __device__ __forceinline__ double cv_f64(TI v) {
    if constexpr (std::is_same_v<TI, __nv_bfloat16>) return (double)__bfloat162float(v);
    else if constexpr (std::is_same_v<TI, __half>) return (double)__half2float(v);
    else return (double)v;
}

template <class TI, class TO, bool TO_BOOL>
__device__ __forceinline__ TO cv_convert(TI v, bool& ok) {
    constexpr bool in_int = std::is_integral_v<TI>;
    constexpr bool out_int = std::is_integral_v<TO>;
    ok = true;
    if constexpr (!out_int) {
        if constexpr (in_int) {
            const long long i = (long long)v;
            if constexpr (std::is_same_v<TO, double>) return __ll2double_rn(i);
            else if constexpr (std::is_same_v<TO, float>) return __ll2float_rn(i);
            else if constexpr (std::is_same_v<TO, __nv_bfloat16>) return __double2bfloat16(__ll2double_rn(i));
            else return __double2half(__ll2double_rn(i));
        } else {
            const double d = cv_f64(v);
            if constexpr (std::is_same_v<TO, double>) return d;
            else if constexpr (std::is_same_v<TO, float>) return __double2float_rn(d);
            else if constexpr (std::is_same_v<TO, __nv_bfloat16>) return __double2bfloat16(d);
            else return __double2half(d);
        }
    } else {
        long long i;
        if constexpr (in_int) {
            i = (long long)v;
        } else {
            const double d = cv_f64(v);
            ok = d == trunc(d) && d >= -9223372036854775808.0 && d < 9223372036854775808.0;
            i = ok ? (long long)d : 0;
        }
        if constexpr (TO_BOOL) ok = ok && (i == 0 || i == 1);
        else if constexpr (std::is_same_v<TO, uint8_t>) ok = ok && i >= 0 && i <= 255;
        else if constexpr (std::is_same_v<TO, int32_t>) ok = ok && i >= INT32_MIN && i <= INT32_MAX;
        return (TO)i;
    }
}

struct ConvertParams {
    const void* src;
    void* dst;
    int64_t sorg, ss1, ss2, dorg, ds1, ds2;
    int64_t n0, n1, rows;
    int* status;
};

template <class TI, class TO, bool TO_BOOL>
__global__ void grid_convert_kernel(const ConvertParams p) {
    const TI* src = (const TI*)p.src;
    TO* dst = (TO*)p.dst;
    bool all_ok = true;
    for (int64_t row = blockIdx.x; row < p.rows; row += gridDim.x) {
        const int64_t y = row % p.n1, z = row / p.n1;
        const TI* s = src + p.sorg + y * p.ss1 + z * p.ss2;
        TO* d = dst + p.dorg + y * p.ds1 + z * p.ds2;
        for (int64_t x = threadIdx.x; x < p.n0; x += blockDim.x) {
            bool ok;
            d[x] = cv_convert<TI, TO, TO_BOOL>(s[x], ok);
            all_ok = all_ok && ok;
        }
    }
    if (!all_ok && p.status) atomicOr(p.status, DEV_ERR_INEXACT);
}

template <class TI>
static int convert_from(const ConvertParams& p, int odt, int blocks, int threads, cudaStream_t s) {
    switch (odt) {
    case STC_F64: grid_convert_kernel<TI, double, false><<<blocks, threads, 0, s>>>(p); break;
    case STC_F32: grid_convert_kernel<TI, float, false><<<blocks, threads, 0, s>>>(p); break;
    case STC_BF16: grid_convert_kernel<TI, __nv_bfloat16, false><<<blocks, threads, 0, s>>>(p); break;
    case STC_F16: grid_convert_kernel<TI, __half, false><<<blocks, threads, 0, s>>>(p); break;
    case STC_U8: grid_convert_kernel<TI, uint8_t, false><<<blocks, threads, 0, s>>>(p); break;
    case STC_BOOL: grid_convert_kernel<TI, uint8_t, true><<<blocks, threads, 0, s>>>(p); break;
    case STC_I32: grid_convert_kernel<TI, int32_t, false><<<blocks, threads, 0, s>>>(p); break;
    case STC_I64: grid_convert_kernel<TI, int64_t, false><<<blocks, threads, 0, s>>>(p); break;
    default: return STC_ERR_UNSUPPORTED;
    }
    return cuda_fail(cudaGetLastError());
}

int launch_grid_convert(const stc_grid* src, int64_t sorg, const stc_grid* dst, int64_t dorg, const int64_t n[3],
                        int* status, cudaStream_t stream) {
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    ConvertParams p{};
    p.src = src->data;
    p.dst = dst->data;
    p.sorg = sorg;
    p.dorg = dorg;
    p.ss1 = src->ndims > 1 ? src->stride[1] : 0;
    p.ss2 = src->ndims > 2 ? src->stride[2] : 0;
    p.ds1 = dst->ndims > 1 ? dst->stride[1] : 0;
    p.ds2 = dst->ndims > 2 ? dst->stride[2] : 0;
    p.n0 = n[0];
    p.n1 = n[1];
    p.rows = n[1] * n[2];
    p.status = status;
    if (p.n0 < 1 || p.rows < 1) return STC_OK;
    const int threads = p.n0 >= 256 ? 256 : 128;
    const int blocks = (int)std::min<int64_t>(p.rows, (int64_t)ctx->num_sms * 16);
    switch (src->dtype) {
    case STC_F64: return convert_from<double>(p, dst->dtype, blocks, threads, stream);
    case STC_F32: return convert_from<float>(p, dst->dtype, blocks, threads, stream);
    case STC_BF16: return convert_from<__nv_bfloat16>(p, dst->dtype, blocks, threads, stream);
    case STC_F16: return convert_from<__half>(p, dst->dtype, blocks, threads, stream);
    case STC_U8: case STC_BOOL: return convert_from<uint8_t>(p, dst->dtype, blocks, threads, stream);
    case STC_I32: return convert_from<int32_t>(p, dst->dtype, blocks, threads, stream);
    case STC_I64: return convert_from<int64_t>(p, dst->dtype, blocks, threads, stream);
    }
    return STC_ERR_UNSUPPORTED;
}

}  // namespace stc
