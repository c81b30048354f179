// float64 and float32 kernels for D = 8, d = 2 (one translation unit per shape so the
// build compiles shapes in parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<8, 2>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 8, 2>::get() : OpsImpl<float, 8, 2>::get();
}
}  // namespace pof
