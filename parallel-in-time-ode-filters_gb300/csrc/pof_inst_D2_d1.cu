// float64 and float32 kernels for D = 2, d = 1 (one translation unit per shape so the
// build compiles shapes in parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<2, 1>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 2, 1>::get() : OpsImpl<float, 2, 1>::get();
}
}  // namespace pof
