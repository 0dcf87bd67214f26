// Generic (offset-table) map kernels for UInt8 / Bool / Int32 / Int64 sources.
#include "map_launch.cuh"

namespace stc {
#define STC_REG_INT(DT, P)                                  \
    static RegisterGeneric<DT, OPV_MEAN> P##0;              \
    static RegisterGeneric<DT, OPV_SUM> P##1;               \
    static RegisterGeneric<DT, OPV_KDOT_D> P##2;            \
    static RegisterGeneric<DT, OPV_MIN> P##3;               \
    static RegisterGeneric<DT, OPV_MAX> P##4;               \
    static RegisterGeneric<DT, OPV_LIFE> P##5;
STC_REG_INT(STC_U8, u)
STC_REG_INT(STC_BOOL, b)
STC_REG_INT(STC_I32, i)
STC_REG_INT(STC_I64, l)
}  // namespace stc
