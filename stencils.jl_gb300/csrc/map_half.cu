// Generic (offset-table) map kernels for BFloat16 / Float16 storage (Float32 accumulation).
#include "map_launch.cuh"

namespace stc {
static RegisterGeneric<STC_BF16, OPV_MEAN> b0;
static RegisterGeneric<STC_BF16, OPV_SUM> b1;
static RegisterGeneric<STC_BF16, OPV_KDOT_D> b2;
static RegisterGeneric<STC_BF16, OPV_KDOT_F> b3;
static RegisterGeneric<STC_BF16, OPV_MIN> b4;
static RegisterGeneric<STC_BF16, OPV_MAX> b5;
static RegisterGeneric<STC_BF16, OPV_DIFFUSE> b6;
static RegisterGeneric<STC_F16, OPV_MEAN> h0;
static RegisterGeneric<STC_F16, OPV_SUM> h1;
static RegisterGeneric<STC_F16, OPV_KDOT_D> h2;
static RegisterGeneric<STC_F16, OPV_KDOT_F> h3;
static RegisterGeneric<STC_F16, OPV_MIN> h4;
static RegisterGeneric<STC_F16, OPV_MAX> h5;
static RegisterGeneric<STC_F16, OPV_DIFFUSE> h6;
}  // namespace stc
