// float64 and float32 kernels for D = 9, d = 3 (one translation unit per shape so the
// build compiles shapes in parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<9, 3>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 9, 3>::get() : OpsImpl<float, 9, 3>::get();
}
}  // namespace pof
