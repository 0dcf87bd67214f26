// Vector-column variants of the 3D shape-specialised map kernels (7-point diffusion, VonNeumann(1)).
// Float32 takes two columns per thread and three CTAs per SM (measured faster than four columns with
// two CTAs on 512^3); 16-bit storage four columns.
#include "map_launch.cuh"

namespace stc {
static RegisterShapeVec<STC_F32, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, 1, 3, 2, 8, 3> w0;
static RegisterShapeVec<STC_BF16, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, 1, 3, 4, 8> w1;
static RegisterShapeVec<STC_F16, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, 1, 3, 4, 8> w1h;
static RegisterShapeVec<STC_F64, OPV_DIFFUSE, STC_SHAPE_VONNEUMANN, 1, 3, 2, 8> w2;
}  // namespace stc
