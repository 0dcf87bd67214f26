// Shape-specialised map kernels: the offset table is a compile-time constant, generated here
// exactly as Stencils.jl generates it, for the configurations the library is tuned for.
// Template arguments: <source type, reduction, shape, R, N, columns/thread, stream slots/thread>.
#include "map_launch.cuh"

namespace stc {
// mean blur, Window(1) 2D (mapstencil(mean, StencilArray(A, Window(1))))
static RegisterShape<STC_F64, OPV_MEAN, STC_SHAPE_WINDOW, 1, 2, 2, 8> s0;
static RegisterShape<STC_F32, OPV_MEAN, STC_SHAPE_WINDOW, 1, 2, 2, 16> s1;
static RegisterShape<STC_BF16, OPV_MEAN, STC_SHAPE_WINDOW, 1, 2, 4, 16> s2;
static RegisterShape<STC_F16, OPV_MEAN, STC_SHAPE_WINDOW, 1, 2, 4, 16> s2h;
// 7x7 kernel, Kernel(Window(3)) 2D, f32 accumulation
static RegisterShape<STC_F32, OPV_KDOT_F, STC_SHAPE_WINDOW, 3, 2, 2, 16> s3;
static RegisterShape<STC_BF16, OPV_KDOT_F, STC_SHAPE_WINDOW, 3, 2, 4, 16> s4;
static RegisterShape<STC_F16, OPV_KDOT_F, STC_SHAPE_WINDOW, 3, 2, 4, 16> s4h;
// 5x5 kernel, Kernel(Window(2)) 2D
static RegisterShape<STC_F32, OPV_KDOT_F, STC_SHAPE_WINDOW, 2, 2, 2, 16> s5;
// Circle(3) mean, Cross(2) sum (2D)
static RegisterShape<STC_F32, OPV_MEAN, STC_SHAPE_CIRCLE, 3, 2, 2, 16> s6;
static RegisterShape<STC_F32, OPV_SUM, STC_SHAPE_CROSS, 2, 2, 2, 16> s7;
// 7-point diffusion, VonNeumann(1) 3D
static RegisterShape<STC_F32, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, 1, 3, 2, 8> s8;
static RegisterShape<STC_BF16, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, 1, 3, 4, 8> s9;
static RegisterShape<STC_F16, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, 1, 3, 4, 8> s9h;
static RegisterShape<STC_F64, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, 1, 3, 2, 8> s10;
// Life on bytes, Moore(1) 2D
static RegisterShape<STC_U8, OPV_LIFE, STC_SHAPE_MOORE, 1, 2, 4, 16> s11;
static RegisterShape<STC_BOOL, OPV_LIFE, STC_SHAPE_MOORE, 1, 2, 4, 16> s12;
}  // namespace stc
