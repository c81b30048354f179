// float64 and float32 kernels for D = 3 with d = 4 observation rows: the Levenberg-Marquardt-regularized model
// of a d = 1, q = 2 problem (the residual row over the D rows of I; pof/observations.py:64-83), used through the
// filter/smoother entry points only (one translation unit per shape so the build compiles shapes in parallel).
#include "pof_table.cuh"

namespace pof {
template <>
const Ops* ops_shape<3, 4>(int dtype) {
  return dtype == 0 ? OpsImpl<double, 3, 4>::get() : OpsImpl<float, 3, 4>::get();
}
}  // namespace pof
