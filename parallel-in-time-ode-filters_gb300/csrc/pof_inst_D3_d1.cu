// float64 and float32 kernels for D = 3, d = 1 (one translation unit per shape so the
// build compiles shapes in parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<3, 1>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 3, 1>::get() : OpsImpl<float, 3, 1>::get();
}
}  // namespace pof
