// float64 and float32 kernels for D = 12, d = 3 (one translation unit per shape so the build compiles shapes in
// parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<12, 3>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 12, 3>::get() : OpsImpl<float, 12, 3>::get();
}
}  // namespace pof
