// Dispatch from runtime (D, d) to the compiled shapes (one translation unit
// per shape: pof_inst_D<D>_d<d>.cu).  d is the number of observation rows:
// d = D / (q + 1) for the EK1 model of an ODE, d > D for the
// Levenberg-Marquardt-regularized model, which only the filter/smoother
// entry points take.
#include "pof_table.cuh"

namespace pof {

#ifdef POF_SHAPE_SUBSET
// The bounds-checked build (pof._build CHECK_SHAPES) compiles the shapes its
// tests run, not all of them.
template <> const Ops* ops_shape<3, 1>(int dtype);
template <> const Ops* ops_shape<8, 2>(int dtype);
template <> const Ops* ops_shape<12, 3>(int dtype);
template <> const Ops* ops_shape<3, 4>(int dtype);

const Ops* find_shape(int dtype, int D, int DY) {
  if (DY < 1 || DY > 9) return nullptr;
  switch (D * 10 + DY) {
    case 31: return ops_shape<3, 1>(dtype);
    case 82: return ops_shape<8, 2>(dtype);
    case 123: return ops_shape<12, 3>(dtype);
    case 34: return ops_shape<3, 4>(dtype);
    default: return nullptr;
  }
}
#else
template <> const Ops* ops_shape<2, 1>(int dtype);
template <> const Ops* ops_shape<3, 1>(int dtype);
template <> const Ops* ops_shape<4, 1>(int dtype);
template <> const Ops* ops_shape<5, 1>(int dtype);
template <> const Ops* ops_shape<6, 1>(int dtype);
template <> const Ops* ops_shape<4, 2>(int dtype);
template <> const Ops* ops_shape<6, 2>(int dtype);
template <> const Ops* ops_shape<8, 2>(int dtype);
template <> const Ops* ops_shape<10, 2>(int dtype);
template <> const Ops* ops_shape<6, 3>(int dtype);
template <> const Ops* ops_shape<9, 3>(int dtype);
template <> const Ops* ops_shape<8, 4>(int dtype);
template <> const Ops* ops_shape<12, 2>(int dtype);
template <> const Ops* ops_shape<12, 3>(int dtype);
template <> const Ops* ops_shape<3, 4>(int dtype);

const Ops* find_shape(int dtype, int D, int DY) {
  if (DY < 1 || DY > 9) return nullptr;
  switch (D * 10 + DY) {
    case 21: return ops_shape<2, 1>(dtype);
    case 31: return ops_shape<3, 1>(dtype);
    case 41: return ops_shape<4, 1>(dtype);
    case 51: return ops_shape<5, 1>(dtype);
    case 61: return ops_shape<6, 1>(dtype);
    case 42: return ops_shape<4, 2>(dtype);
    case 62: return ops_shape<6, 2>(dtype);
    case 82: return ops_shape<8, 2>(dtype);
    case 102: return ops_shape<10, 2>(dtype);
    case 63: return ops_shape<6, 3>(dtype);
    case 93: return ops_shape<9, 3>(dtype);
    case 84: return ops_shape<8, 4>(dtype);
    case 122: return ops_shape<12, 2>(dtype);
    case 123: return ops_shape<12, 3>(dtype);
    case 34: return ops_shape<3, 4>(dtype);  // more observation rows than states (LM-regularized model)
    default: return nullptr;
  }
}

#endif

}  // namespace pof
