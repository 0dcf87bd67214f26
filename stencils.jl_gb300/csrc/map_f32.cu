// Generic (offset-table) map kernels for Float32 sources.
#include "map_launch.cuh"

namespace stc {
static RegisterGeneric<STC_F32, OPV_MEAN> r0;
static RegisterGeneric<STC_F32, OPV_SUM> r1;
static RegisterGeneric<STC_F32, OPV_KDOT_D> r2;
static RegisterGeneric<STC_F32, OPV_KDOT_F> r3;
static RegisterGeneric<STC_F32, OPV_MIN> r4;
static RegisterGeneric<STC_F32, OPV_MAX> r5;
static RegisterGeneric<STC_F32, OPV_DIFFUSE> r6;
}  // namespace stc
