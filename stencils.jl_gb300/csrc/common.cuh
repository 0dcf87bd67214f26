// common.cuh — element traits, exact arithmetic helpers, bounded mbarrier / TMA primitives.
//
// All floating-point arithmetic on the parity path uses explicit round-to-nearest intrinsics
// (__dadd_rn, __dmul_rn, ...) so that nvcc cannot contract `s + a*b` into an FMA: the reference
// (Julia) evaluates the multiply and the add separately.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/stencil_cuda.h"

namespace stc {

// ------------------------------------------------------------------ status word
// Kernels that give up a bounded wait OR a bit into this word; the host reads and clears it.
enum : int { DEV_ERR_TIMEOUT = 1, DEV_ERR_BOUNDS = 2, DEV_ERR_INEXACT = 4 };

// Debug builds (-DSTC_DEBUG_BOUNDS: `build.py --debug`, libstencilcuda_debug.so): kernels test the indices
// of their computed shared-memory accesses against the buffers they address before making them.  An index
// out of range skips the access and ORs DEV_ERR_BOUNDS into the launch's status slot — never a trap — so the
// host call returns STC_ERR_BOUNDS.  Release builds compile the tests out.
#ifdef STC_DEBUG_BOUNDS
__device__ __forceinline__ bool bounds_ok(int64_t i, int64_t n, int* status) {
    if (i >= 0 && i < n) return true;
    if (status) atomicOr(status, DEV_ERR_BOUNDS);
    return false;
}
#define STC_IN_BOUNDS(i, n, status) ::stc::bounds_ok((int64_t)(i), (int64_t)(n), (status))
#else
#define STC_IN_BOUNDS(i, n, status) true
#endif

// ------------------------------------------------------------------ element traits
template <int DT> struct Elem;
template <> struct Elem<STC_F64>  { using T = double;          static constexpr bool is_float = true; };
template <> struct Elem<STC_F32>  { using T = float;           static constexpr bool is_float = true; };
template <> struct Elem<STC_BF16> { using T = __nv_bfloat16;   static constexpr bool is_float = true; };
template <> struct Elem<STC_F16>  { using T = __half;          static constexpr bool is_float = true; };
template <> struct Elem<STC_U8>   { using T = uint8_t;         static constexpr bool is_float = false; };
template <> struct Elem<STC_BOOL> { using T = uint8_t;         static constexpr bool is_float = false; };
template <> struct Elem<STC_I32>  { using T = int32_t;         static constexpr bool is_float = false; };
template <> struct Elem<STC_I64>  { using T = int64_t;         static constexpr bool is_float = false; };

__device__ __forceinline__ double cvt_d(double x) { return x; }
__device__ __forceinline__ double cvt_d(float x) { return (double)x; }
__device__ __forceinline__ double cvt_d(__nv_bfloat16 x) { return (double)__bfloat162float(x); }
__device__ __forceinline__ double cvt_d(__half x) { return (double)__half2float(x); }
__device__ __forceinline__ double cvt_d(uint8_t x) { return (double)x; }
__device__ __forceinline__ double cvt_d(int32_t x) { return (double)x; }
__device__ __forceinline__ double cvt_d(int64_t x) { return (double)x; }

__device__ __forceinline__ float cvt_f(float x) { return x; }
__device__ __forceinline__ float cvt_f(__nv_bfloat16 x) { return __bfloat162float(x); }
__device__ __forceinline__ float cvt_f(__half x) { return __half2float(x); }

__device__ __forceinline__ int64_t cvt_i(uint8_t x) { return (int64_t)x; }
__device__ __forceinline__ int64_t cvt_i(int32_t x) { return (int64_t)x; }
__device__ __forceinline__ int64_t cvt_i(int64_t x) { return x; }

// accumulator -> stored element (round to nearest even)
template <class T> __device__ __forceinline__ T from_f64(double x);
template <> __device__ __forceinline__ double from_f64<double>(double x) { return x; }
template <> __device__ __forceinline__ float from_f64<float>(double x) { return __double2float_rn(x); }
template <class T> __device__ __forceinline__ T from_f32(float x);
template <> __device__ __forceinline__ float from_f32<float>(float x) { return x; }
template <> __device__ __forceinline__ double from_f32<double>(float x) { return (double)x; }
template <> __device__ __forceinline__ __nv_bfloat16 from_f32<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <> __device__ __forceinline__ __half from_f32<__half>(float x) { return __float2half_rn(x); }

// Julia's min/max on floats: NaN-propagating, -0.0 ordered below +0.0.
__device__ __forceinline__ double jl_min(double x, double y) {
    if (isnan(x) || isnan(y)) return __longlong_as_double(0x7ff8000000000000ll);
    return (x < y || (x == y && signbit(x))) ? x : y;
}
__device__ __forceinline__ double jl_max(double x, double y) {
    if (isnan(x) || isnan(y)) return __longlong_as_double(0x7ff8000000000000ll);
    return (x > y || (x == y && !signbit(x))) ? x : y;
}
__device__ __forceinline__ float jl_min(float x, float y) {
    if (isnan(x) || isnan(y)) return __int_as_float(0x7fc00000);
    return (x < y || (x == y && signbit(x))) ? x : y;
}
__device__ __forceinline__ float jl_max(float x, float y) {
    if (isnan(x) || isnan(y)) return __int_as_float(0x7fc00000);
    return (x > y || (x == y && !signbit(x))) ? x : y;
}

// integer wrap to the width of an element type (sum of UInt8 wraps mod 256, Int32 mod 2^32)
template <int DT> __device__ __forceinline__ int64_t wrap_int(int64_t x) {
    if constexpr (DT == STC_U8 || DT == STC_BOOL) return (int64_t)(uint8_t)x;
    else if constexpr (DT == STC_I32) return (int64_t)(int32_t)(uint32_t)(uint64_t)x;
    else return x;
}

// ------------------------------------------------------------------ smem / mbarrier / TMA
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void fence_barrier_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// try_wait with a suspend-time hint: the thread sleeps in hardware until the phase completes or
// the hint (nanoseconds) elapses, instead of spinning through issue slots.
__device__ __forceinline__ bool mbar_try_wait_sleep(uint64_t* bar, uint32_t parity, uint32_t hint_ns) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity), "r"(hint_ns)
        : "memory");
    return ok != 0;
}

// Bounded wait: gives up after ~`limit_cycles` SM clocks and reports false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity,
                                                  long long limit_cycles = 4000000000ll) {
    if (mbar_try_wait(bar, parity)) return true;
    const long long t0 = clock64();
    while (true) {
        if (mbar_try_wait_sleep(bar, parity, 20000u)) return true;
        if (clock64() - t0 > limit_cycles) return false;
    }
}

// TMA tiled loads (no multicast: every CTA reads its own tile of this GPU's memory)
__device__ __forceinline__ void tma_load_1d(void* dst, const CUtensorMap* tm, uint64_t* bar, int x) {
    asm volatile(
        "cp.async.bulk.tensor.1d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];"
        ::"r"(smem_u32(dst)), "l"(tm), "r"(x), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(tm), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* tm, uint64_t* bar, int x, int y,
                                            int z) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(smem_u32(dst)), "l"(tm), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void prefetch_tensormap(const CUtensorMap* tm) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(tm) : "memory");
}

}  // namespace stc
