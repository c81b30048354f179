// Batched-solve kernels for D = 6, d = 2, float64 and float32 (one
// translation unit per shape so the build compiles shapes in parallel).
#include "pof_batch.cuh"

namespace pof {
template <>
const BatchOps* batch_ops_shape<6, 2>(int dtype) {
  return dtype == 0 ? batch_ops_impl<double, 6, 2>() : batch_ops_impl<float, 6, 2>();
}
}  // namespace pof
