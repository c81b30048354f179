// Strided matrix views of the dense path (shared by the CUDA kernels, the
// schedule and its host-side check).
#pragma once

#include <stdint.h>

#ifdef __CUDACC__
#define POF_DHD __host__ __device__
#else
#define POF_DHD
#endif

namespace pof {
namespace dense {

// Matrix view: element (b, i, j) at p[b * bs + i * rs + j * cs].
template <typename T>
struct MV {
  T* p;
  int64_t rs, cs, bs;
};

template <typename T>
POF_DHD inline MV<T> tr(MV<T> a) {
  return MV<T>{a.p, a.cs, a.rs, a.bs};
}
template <typename T>
POF_DHD inline MV<T> sub(MV<T> a, int64_t i, int64_t j) {
  return MV<T>{a.p + i * a.rs + j * a.cs, a.rs, a.cs, a.bs};
}
// Row-major matrices with `cols` columns, `bs` elements apart.
template <typename T>
inline MV<T> rowmajor(T* p, int64_t cols, int64_t bs) {
  return MV<T>{p, cols, 1, bs};
}

// Rows of a tria panel (the reflectors of one panel kernel), at most.
constexpr int kMaxPanel = 32;

}  // namespace dense
}  // namespace pof
