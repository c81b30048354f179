// float64 and float32 kernels for D = 4, d = 2 (one translation unit per shape so the
// build compiles shapes in parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<4, 2>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 4, 2>::get() : OpsImpl<float, 4, 2>::get();
}
}  // namespace pof
