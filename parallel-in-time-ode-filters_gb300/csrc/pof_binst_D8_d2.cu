// Batched-solve kernels for D = 8, d = 2, float64 and float32 (one
// translation unit per shape so the build compiles shapes in parallel).
#include "pof_batch.cuh"

namespace pof {
template <>
const BatchOps* batch_ops_shape<8, 2>(int dtype) {
  return dtype == 0 ? batch_ops_impl<double, 8, 2>() : batch_ops_impl<float, 8, 2>();
}
}  // namespace pof
