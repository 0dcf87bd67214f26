// Vector-column variants (XV adjacent columns per thread, aligned vector shared-memory loads and
// global stores) of the 2D shape-specialised map kernels.  Template arguments: <source type,
// reduction, shape, R, N, columns per thread, stream slots per thread>.
#include "map_launch.cuh"

namespace stc {
// 7x7 and 5x5 kernels, f32 accumulation
static RegisterShapeVec<STC_F32, OPV_KDOT_F, STC_SHAPE_WINDOW, 3, 2, 4, 8> v0;
static RegisterShapeVec<STC_BF16, OPV_KDOT_F, STC_SHAPE_WINDOW, 3, 2, 4, 8> v1;
static RegisterShapeVec<STC_F16, OPV_KDOT_F, STC_SHAPE_WINDOW, 3, 2, 4, 8> v1h;
static RegisterShapeVec<STC_F32, OPV_KDOT_F, STC_SHAPE_WINDOW, 2, 2, 4, 8> v2;
// mean blur Window(1); Float64 on 64 x 16 tiles (2 stream rows per warp): the FP64 map of a 1000^2 grid is
// latency-bound, and more, smaller tiles per SM measured 26.8 us per map against 29.9 us with 64 x 32 tiles
// and 35.7 us with 64 x 64
static RegisterShapeVec<STC_F64, OPV_MEAN, STC_SHAPE_WINDOW, 1, 2, 2, 2> v3;
static RegisterShapeVec<STC_F32, OPV_MEAN, STC_SHAPE_WINDOW, 1, 2, 4, 8> v4;
static RegisterShapeVec<STC_BF16, OPV_MEAN, STC_SHAPE_WINDOW, 1, 2, 4, 8> v5;
static RegisterShapeVec<STC_F16, OPV_MEAN, STC_SHAPE_WINDOW, 1, 2, 4, 8> v5h;
// Circle(3) mean, Cross(2) sum
static RegisterShapeVec<STC_F32, OPV_MEAN, STC_SHAPE_CIRCLE, 3, 2, 4, 8> v6;
static RegisterShapeVec<STC_F32, OPV_SUM, STC_SHAPE_CROSS, 2, 2, 4, 8> v7;
// Life on bytes, Moore(1)
static RegisterShapeVec<STC_U8, OPV_LIFE, STC_SHAPE_MOORE, 1, 2, 4, 16> v8;
static RegisterShapeVec<STC_BOOL, OPV_LIFE, STC_SHAPE_MOORE, 1, 2, 4, 16> v9;
}  // namespace stc
