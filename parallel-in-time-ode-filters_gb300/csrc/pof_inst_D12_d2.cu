// float64 and float32 kernels for D = 12, d = 2 (one translation unit per shape so the build compiles shapes in
// parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<12, 2>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 12, 2>::get() : OpsImpl<float, 12, 2>::get();
}
}  // namespace pof
