// Dispatch from runtime (D, d) to the compiled batch shapes (one
// translation unit per shape: pof_binst_D<D>_d<d>.cu).
#include "pof_batch.cuh"

namespace pof {

#ifdef POF_SHAPE_SUBSET
// the bounds-checked build's shapes (pof._build CHECK_SHAPES)
template <> const BatchOps* batch_ops_shape<8, 2>(int dtype);

const BatchOps* find_batch_shape(int dtype, int D, int DY) {
  if (dtype != 0 && dtype != 1) return nullptr;
  return D * 10 + DY == 82 ? batch_ops_shape<8, 2>(dtype) : nullptr;
}
#else
template <> const BatchOps* batch_ops_shape<3, 1>(int dtype);
template <> const BatchOps* batch_ops_shape<4, 1>(int dtype);
template <> const BatchOps* batch_ops_shape<5, 1>(int dtype);
template <> const BatchOps* batch_ops_shape<6, 2>(int dtype);
template <> const BatchOps* batch_ops_shape<8, 2>(int dtype);
template <> const BatchOps* batch_ops_shape<10, 2>(int dtype);

const BatchOps* find_batch_shape(int dtype, int D, int DY) {
  if (dtype != 0 && dtype != 1) return nullptr;
  switch (D * 10 + DY) {
    case 31: return batch_ops_shape<3, 1>(dtype);
    case 41: return batch_ops_shape<4, 1>(dtype);
    case 51: return batch_ops_shape<5, 1>(dtype);
    case 62: return batch_ops_shape<6, 2>(dtype);
    case 82: return batch_ops_shape<8, 2>(dtype);
    case 102: return batch_ops_shape<10, 2>(dtype);
    default: return nullptr;
  }
}

#endif

}  // namespace pof
