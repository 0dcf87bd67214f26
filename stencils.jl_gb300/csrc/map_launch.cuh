// map_launch.cuh — host launchers for the map kernels, the element/op type table, and the
// registration helpers each instantiation unit uses.
#pragma once

#include <atomic>
#include <mutex>

#include "dispatch.h"
#include "map_kernel.cuh"

namespace stc {

// Per-output gather straight from global memory (L1/L2 cached), boundary rules per access.  Used
// only when a tile plus its halo does not fit in shared memory (very large radii).
template <class Tin, class Tout, class Op>
__global__ void __launch_bounds__(256) map_direct_kernel(const __grid_constant__ MapParams p) {
    const int64_t total = p.n[0] * p.n[1] * p.n[2];
    Tout* dst = (Tout*)p.dst;
    for (int64_t lin = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; lin < total;
         lin += (int64_t)gridDim.x * blockDim.x) {
        const int64_t x = lin % p.n[0], r = lin / p.n[0];
        const int64_t y = r % p.n[1], z = r / p.n[1];
        typename Op::A a;
        int k0 = 0;
        if constexpr (Op::kZeroInit) {
            a = Op::first(Tin(0), 0);
        } else {
            a = Op::first(load_bounded<Tin>(p, x + p.off[0][0], y + p.off[0][1], z + p.off[0][2]), 0);
            k0 = 1;
        }
        for (int k = k0; k < p.L; ++k)
            a = Op::step(a, load_bounded<Tin>(p, x + p.off[k][0], y + p.off[k][1], z + p.off[k][2]), k, p);
        dst[p.dst_org + x + y * p.dstr[1] + z * p.dstr[2]] = Op::finish(a, load_bounded<Tin>(p, x, y, z), p);
    }
}

struct TableShape { static constexpr int kKind = STC_SHAPE_TABLE, kR = 0, kN = 0, L = 0; };

// occupancy per (kernel, dynamic smem) is cached; cudaFuncSetAttribute is raised once per size
struct LaunchCache {
    std::mutex mu;
    size_t smem_set = 48 * 1024;
    size_t occ_smem[8] = {0};
    int occ_val[8] = {0};
    int occ_n = 0;
};

template <class K>
static cudaError_t prepare_launch(K kern, LaunchCache& c, size_t smem, int* per_sm) {
    std::lock_guard<std::mutex> g(c.mu);
    if (smem > c.smem_set) {
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        c.smem_set = smem;
    }
    for (int i = 0; i < c.occ_n; ++i)
        if (c.occ_smem[i] == smem) { *per_sm = c.occ_val[i]; return cudaSuccess; }
    int v = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v, kern, kMapThreads, smem);
    if (e != cudaSuccess) return e;
    if (c.occ_n < 8) { c.occ_smem[c.occ_n] = smem; c.occ_val[c.occ_n] = v; ++c.occ_n; }
    *per_sm = v;
    return cudaSuccess;
}

template <class Tin, class Tout, class Op, class Sh, int XT, int VS, bool VEC = false, int MINB = 2>
cudaError_t launch_tiled(MapParams& p, cudaStream_t stream, int num_sms) {
    static LaunchCache cache;
    // only the variant this launcher runs is instantiated
    void (*kern)(const MapParams);
    if constexpr (VEC) kern = map_vec_kernel<Tin, Tout, Op, Sh, XT, VS, MINB>;
    else kern = map_kernel<Tin, Tout, Op, Sh, XT, VS>;
    const size_t smem = (size_t)(p.use_tma ? p.stages : 1) * p.stage_bytes + (size_t)kMaxStages * 8;
    int per_sm = 0;
    cudaError_t e = prepare_launch(kern, cache, smem, &per_sm);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) return cudaErrorInvalidConfiguration;
    int64_t grid = (int64_t)per_sm * num_sms;
    if (grid > p.ntiles) grid = p.ntiles;
    if (grid < 1) return cudaSuccess;
    kern<<<(unsigned)grid, kMapThreads, smem, stream>>>(p);
    return cudaGetLastError();
}

template <class Tin, class Tout, class Op>
cudaError_t launch_direct(MapParams& p, cudaStream_t stream, int num_sms) {
    const int64_t total = p.n[0] * p.n[1] * p.n[2];
    if (total == 0) return cudaSuccess;
    int64_t grid = (total + 255) / 256;
    if (grid > (int64_t)num_sms * 16) grid = (int64_t)num_sms * 16;
    map_direct_kernel<Tin, Tout, Op><<<(unsigned)grid, 256, 0, stream>>>(p);
    return cudaGetLastError();
}

// ---------------------------------------------------------------------------- type table
template <int DT, int OPV> struct OpFor;

#define STC_FLOAT_OPS(DT, TIN, ACC)                                                             \
    template <> struct OpFor<DT, OPV_MEAN> { using Tin = TIN; using Tout = TIN; using Op = OpMean<TIN, TIN, ACC>; }; \
    template <> struct OpFor<DT, OPV_SUM> { using Tin = TIN; using Tout = TIN; using Op = OpSumF<TIN, TIN, ACC>; }; \
    template <> struct OpFor<DT, OPV_MIN> { using Tin = TIN; using Tout = TIN; using Op = OpMinMaxF<TIN, TIN, ACC, false>; }; \
    template <> struct OpFor<DT, OPV_MAX> { using Tin = TIN; using Tout = TIN; using Op = OpMinMaxF<TIN, TIN, ACC, true>; }; \
    template <> struct OpFor<DT, OPV_DIFFUSE> { using Tin = TIN; using Tout = TIN; using Op = OpDiffuse<TIN, TIN, ACC>; }; \
    template <> struct OpFor<DT, OPV_KDOT_D> { using Tin = TIN; using Tout = double; using Op = OpKdotD<TIN, double>; };

STC_FLOAT_OPS(STC_F64, double, double)
STC_FLOAT_OPS(STC_F32, float, float)
STC_FLOAT_OPS(STC_BF16, __nv_bfloat16, float)
STC_FLOAT_OPS(STC_F16, __half, float)
template <> struct OpFor<STC_F32, OPV_KDOT_F> { using Tin = float; using Tout = float; using Op = OpKdotF<float, float>; };
template <> struct OpFor<STC_BF16, OPV_KDOT_F> { using Tin = __nv_bfloat16; using Tout = __nv_bfloat16; using Op = OpKdotF<__nv_bfloat16, __nv_bfloat16>; };
template <> struct OpFor<STC_F16, OPV_KDOT_F> { using Tin = __half; using Tout = __half; using Op = OpKdotF<__half, __half>; };

#define STC_INT_OPS(DT, TIN, SUMOUT, SUMACC)                                                      \
    template <> struct OpFor<DT, OPV_MEAN> { using Tin = TIN; using Tout = double; using Op = OpMean<TIN, double, double>; }; \
    template <> struct OpFor<DT, OPV_SUM> { using Tin = TIN; using Tout = SUMOUT; using Op = OpSumI<TIN, SUMOUT, SUMACC>; }; \
    template <> struct OpFor<DT, OPV_MIN> { using Tin = TIN; using Tout = TIN; using Op = OpMinMaxI<TIN, TIN, false>; }; \
    template <> struct OpFor<DT, OPV_MAX> { using Tin = TIN; using Tout = TIN; using Op = OpMinMaxI<TIN, TIN, true>; }; \
    template <> struct OpFor<DT, OPV_LIFE> { using Tin = TIN; using Tout = TIN; using Op = OpLife<TIN, TIN>; }; \
    template <> struct OpFor<DT, OPV_KDOT_D> { using Tin = TIN; using Tout = double; using Op = OpKdotD<TIN, double>; };

STC_INT_OPS(STC_U8, uint8_t, uint8_t, STC_U8)
STC_INT_OPS(STC_BOOL, uint8_t, int64_t, STC_I64)
STC_INT_OPS(STC_I32, int32_t, int32_t, STC_I32)
STC_INT_OPS(STC_I64, int64_t, int64_t, STC_I64)

// generic tile geometry per element size: (columns per thread, slots per thread)
template <class T> struct GenericTile { static constexpr int XT = sizeof(T) >= 4 ? 2 : 4; static constexpr int VS = sizeof(T) == 8 ? 4 : 8; };

template <int DT, int OPV>
struct RegisterGeneric {
    RegisterGeneric() {
        using F = OpFor<DT, OPV>;
        using G = GenericTile<typename F::Tin>;
        KernelEntry e;
        e.launch = &launch_tiled<typename F::Tin, typename F::Tout, typename F::Op, TableShape, G::XT, G::VS>;
        e.launch_direct = &launch_direct<typename F::Tin, typename F::Tout, typename F::Op>;
        e.xt = G::XT;
        e.vs = G::VS;
        register_kernel(DT, OPV, STC_SHAPE_TABLE, 0, 0, e);
    }
};

template <int DT, int OPV, int KIND, int R, int N, int XT, int VS>
struct RegisterShape {
    RegisterShape() {
        using F = OpFor<DT, OPV>;
        KernelEntry e;
        e.launch = &launch_tiled<typename F::Tin, typename F::Tout, typename F::Op, Shape<KIND, R, N>, XT, VS>;
        e.xt = XT;
        e.vs = VS;
        e.kind = KIND;
        e.R = R;
        e.N = N;
        register_kernel(DT, OPV, KIND, R, N, e);
    }
};

// The vector-column variant of a shape kernel (XV adjacent columns per thread); launch_map uses it
// when the tile's first column lands on an XV-aligned shared-memory index, else the variant above.
template <int DT, int OPV, int KIND, int R, int N, int XV, int VS, int MINB = 2>
struct RegisterShapeVec {
    RegisterShapeVec() {
        using F = OpFor<DT, OPV>;
        static_assert(XV * sizeof(typename F::Tin) <= 16, "one vector load per XV columns");
        KernelEntry e;
        e.launch_vec = &launch_tiled<typename F::Tin, typename F::Tout, typename F::Op, Shape<KIND, R, N>, XV, VS, true, MINB>;
        e.xv = XV;
        e.vs_vec = VS;
        e.kind = KIND;
        e.R = R;
        e.N = N;
        register_kernel(DT, OPV, KIND, R, N, e);
    }
};

}  // namespace stc
