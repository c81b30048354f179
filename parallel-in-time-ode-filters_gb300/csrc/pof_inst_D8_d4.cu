// float64 and float32 kernels for D = 8, d = 4 (one translation unit per shape so the
// build compiles shapes in parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<8, 4>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 8, 4>::get() : OpsImpl<float, 8, 4>::get();
}
}  // namespace pof
