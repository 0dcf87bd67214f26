// Generic (offset-table) map kernels for Float64 sources.
#include "map_launch.cuh"

namespace stc {
static RegisterGeneric<STC_F64, OPV_MEAN> r0;
static RegisterGeneric<STC_F64, OPV_SUM> r1;
static RegisterGeneric<STC_F64, OPV_KDOT_D> r2;
static RegisterGeneric<STC_F64, OPV_MIN> r3;
static RegisterGeneric<STC_F64, OPV_MAX> r4;
static RegisterGeneric<STC_F64, OPV_DIFFUSE> r5;
}  // namespace stc
