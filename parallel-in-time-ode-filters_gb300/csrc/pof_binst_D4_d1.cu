// Batched-solve kernels for D = 4, d = 1, float64 and float32 (one
// translation unit per shape so the build compiles shapes in parallel).
#include "pof_batch.cuh"

namespace pof {
template <>
const BatchOps* batch_ops_shape<4, 1>(int dtype) {
  return dtype == 0 ? batch_ops_impl<double, 4, 1>() : batch_ops_impl<float, 4, 1>();
}
}  // namespace pof
