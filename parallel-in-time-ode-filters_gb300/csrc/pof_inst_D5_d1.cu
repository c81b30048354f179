// float64 and float32 kernels for D = 5, d = 1 (one translation unit per shape so the
// build compiles shapes in parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<5, 1>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 5, 1>::get() : OpsImpl<float, 5, 1>::get();
}
}  // namespace pof
