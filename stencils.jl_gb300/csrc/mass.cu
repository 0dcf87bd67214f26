// mass.cu — K4: FP64 total of a grid with Neumaier compensation, for the mass-drift report of
// long multi-step runs (no counterpart in the reference; the oracle's orc_mass is its checker).
//
// Each thread accumulates a compensated (sum, correction) pair over a grid-stride walk of the
// logical cells; pairs are combined with the same compensated addition across the warp, the block
// and finally across blocks (one partial per block in a device scratch buffer).
#include <mutex>

#include "common.cuh"
#include "dispatch.h"

namespace stc {

struct CPair { double s, c; };

__device__ __forceinline__ CPair cadd(CPair a, double x) {
    const double t = a.s + x;
    if (fabs(a.s) >= fabs(x)) a.c += (a.s - t) + x;
    else a.c += (x - t) + a.s;
    a.s = t;
    return a;
}
__device__ __forceinline__ CPair ccombine(CPair a, CPair b) {
    a = cadd(a, b.s);
    a.c += b.c;
    return a;
}

struct MassParams {
    const void* base;
    int64_t st[3];
    int64_t n[3];
    int64_t org;
};

template <class T>
__device__ __forceinline__ CPair block_reduce(CPair v) {
    __shared__ CPair sh[32];
    for (int o = 16; o > 0; o >>= 1) {
        CPair w;
        w.s = __shfl_down_sync(0xffffffffu, v.s, o);
        w.c = __shfl_down_sync(0xffffffffu, v.c, o);
        v = ccombine(v, w);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) sh[warp] = v;
    __syncthreads();
    if (warp == 0) {
        const int nw = (blockDim.x + 31) / 32;
        v = lane < nw ? sh[lane] : CPair{0.0, 0.0};
        for (int o = 16; o > 0; o >>= 1) {
            CPair w;
            w.s = __shfl_down_sync(0xffffffffu, v.s, o);
            w.c = __shfl_down_sync(0xffffffffu, v.c, o);
            v = ccombine(v, w);
        }
    }
    return v;
}

template <class T>
__global__ void __launch_bounds__(256) mass_partial_kernel(const MassParams p, CPair* partial) {
    const T* base = (const T*)p.base;
    const int64_t total = p.n[0] * p.n[1] * p.n[2];
    CPair acc{0.0, 0.0};
    for (int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lin < total;
         lin += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = lin % p.n[0], r = lin / p.n[0];
        const int64_t y = r % p.n[1], z = r / p.n[1];
        acc = cadd(acc, cvt_d(base[p.org + x + y * p.st[1] + z * p.st[2]]));
    }
    acc = block_reduce<T>(acc);
    if (threadIdx.x == 0) partial[blockIdx.x] = acc;
}

__global__ void __launch_bounds__(256) mass_final_kernel(const CPair* partial, int n, double* out) {
    CPair acc{0.0, 0.0};
    for (int i = threadIdx.x; i < n; i += blockDim.x) acc = ccombine(acc, partial[i]);
    acc = block_reduce<double>(acc);
    if (threadIdx.x == 0) out[0] = acc.s + acc.c;
}

// per-device scratch: partial pairs + the result
static std::mutex g_mass_mu;
static void* g_mass_scratch[64] = {nullptr};

int mass_launch(const stc_grid* g, int radius, const stc_bc* bc, double* dev_out, CPair* partial, int nblocks,
                cudaStream_t s);

int mass_launch(const stc_grid* g, int radius, const stc_bc* bc, double* dev_out, CPair* partial, int nblocks,
                cudaStream_t s) {
    MassParams p{};
    const bool halo = bc && bc->padding != STC_CONDITIONAL;
    p.base = g->data;
    for (int d = 0; d < 3; ++d) {
        p.n[d] = d < g->ndims ? g->size[d] - (halo ? 2 * radius : 0) : 1;
        p.st[d] = d < g->ndims ? g->stride[d] : 0;
        if (halo && d < g->ndims) p.org += (int64_t)radius * g->stride[d];
        if (p.n[d] < 0) return STC_ERR_RADIUS;
    }
    switch (g->dtype) {
    case STC_F64: mass_partial_kernel<double><<<nblocks, 256, 0, s>>>(p, partial); break;
    case STC_F32: mass_partial_kernel<float><<<nblocks, 256, 0, s>>>(p, partial); break;
    case STC_BF16: mass_partial_kernel<__nv_bfloat16><<<nblocks, 256, 0, s>>>(p, partial); break;
    case STC_F16: mass_partial_kernel<__half><<<nblocks, 256, 0, s>>>(p, partial); break;
    case STC_U8: case STC_BOOL: mass_partial_kernel<uint8_t><<<nblocks, 256, 0, s>>>(p, partial); break;
    case STC_I32: mass_partial_kernel<int32_t><<<nblocks, 256, 0, s>>>(p, partial); break;
    case STC_I64: mass_partial_kernel<int64_t><<<nblocks, 256, 0, s>>>(p, partial); break;
    default: return STC_ERR_UNSUPPORTED;
    }
    mass_final_kernel<<<1, 256, 0, s>>>(partial, nblocks, dev_out);
    return cuda_fail(cudaGetLastError());
}

}  // namespace stc

using namespace stc;

extern "C" int stc_mass(const stc_grid* g, int32_t radius, const stc_bc* bc, double* out_total, void* stream) {
    if (!g || !out_total || g->ndims < 1 || g->ndims > 3 || dtype_size(g->dtype) == 0 || radius < 0)
        return STC_ERR_INVALID;
    DeviceCtx* ctx = nullptr;
    int rc = device_ctx(&ctx);
    if (rc) return rc;
    const int nblocks = ctx->num_sms * 4;
    void* scratch;
    {
        std::lock_guard<std::mutex> lk(g_mass_mu);
        if (!g_mass_scratch[ctx->device]) {
            cudaError_t e = cudaMalloc(&g_mass_scratch[ctx->device], sizeof(CPair) * (nblocks + 1));
            if (e != cudaSuccess) return cuda_fail(e);
        }
        scratch = g_mass_scratch[ctx->device];
    }
    cudaStream_t s = (cudaStream_t)stream;
    CPair* partial = (CPair*)scratch;
    double* dev_out = (double*)(partial + nblocks);
    if ((rc = mass_launch(g, radius, bc, dev_out, partial, nblocks, s))) return rc;
    cudaError_t e = cudaMemcpyAsync(out_total, dev_out, sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e != cudaSuccess) return cuda_fail(e);
    return cuda_fail(cudaStreamSynchronize(s));
}
