// Type-erased table of the driver for one (dtype, D, DY), so the C ABI can
// dispatch on runtime sizes while every kernel is compiled for fixed sizes.
#pragma once

#include <cuda_runtime.h>

#include "pof_driver.cuh"
#include "pof_seq.cuh"

namespace pof {

struct Ops {
  void (*filter)(const Plan&, char*, const StepModel&, const void*, const void*, void*, void*, cudaStream_t);
  void (*smoother)(const Plan&, char*, const void*, const void*, int64_t, void*, void*, bool, const void*,
                   cudaStream_t);
  void (*smo_elements)(int64_t, const void*, const void*, int64_t, const void*, const void*, void*, cudaStream_t);
  void (*linearize)(int64_t, int, const void*, double, double, const void*, void*, void*, cudaStream_t);
  void (*scale_inplace)(void*, int64_t, const void*, cudaStream_t);
  void (*sequential)(int64_t, const StepModel&, int, const void*, double, double, const void*, const void*, int,
                     void*, void*, double*, cudaStream_t);
};

template <typename T, int D, int DY>
struct OpsImpl {
  static void filter(const Plan& p, char* ws, const StepModel& sm, const void* x0m, const void* x0L, void* means,
                     void* chols, cudaStream_t st) {
    Driver<T, D, DY>::filter(p, ws, sm, static_cast<const T*>(x0m), static_cast<const T*>(x0L),
                             static_cast<T*>(means), static_cast<T*>(chols), st);
  }
  static void smoother(const Plan& p, char* ws, const void* F, const void* QL, int64_t fts, void* means,
                       void* chols, bool calibrate, const void* means_old, cudaStream_t st) {
    Driver<T, D, DY>::smoother(p, ws, static_cast<const T*>(F), static_cast<const T*>(QL), fts,
                               static_cast<T*>(means), static_cast<T*>(chols), calibrate,
                               static_cast<const T*>(means_old), st);
  }
  static void smo_elements(int64_t n, const void* F, const void* QL, int64_t fts, const void* fm, const void* fL,
                           void* selems, cudaStream_t st) {
    k_smo_elements<T, D><<<grid_for(n, 64), 64, 0, st>>>(n, static_cast<const T*>(F), static_cast<const T*>(QL),
                                                         fts, static_cast<const T*>(fm),
                                                         static_cast<const T*>(fL), static_cast<T*>(selems));
  }
  static void linearize(int64_t n, int field, const void* params, double p0, double p1, const void* means, void* H,
                        void* c, cudaStream_t st) {
    // a field's EK1 model has d = D / (q + 1) rows; shapes with more rows
    // than states exist for given (H, c, R) only and never get here
    if constexpr (D % DY == 0)
      Driver<T, D, DY>::linearize(n, field, static_cast<const T*>(params), (T)p0, (T)p1,
                                  static_cast<const T*>(means), static_cast<T*>(H), static_cast<T*>(c), st);
  }
  static void scale_inplace(void* x, int64_t count, const void* scale, cudaStream_t st) {
    k_scale_inplace<T><<<grid_for(count, 256), 256, 0, st>>>(static_cast<T*>(x), count,
                                                             static_cast<const T*>(scale));
  }
  static void sequential(int64_t n, const StepModel& sm, int field, const void* params, double p0, double p1,
                         const void* x0m, const void* x0L, int smooth, void* means, void* chols, double* scalars,
                         cudaStream_t st) {
    ProfScope ps(PK_SEQUENTIAL, st);
    k_seq_filtsmooth<T, D, DY><<<1, 32, 0, st>>>(n, sm, field, static_cast<const T*>(params), (T)p0, (T)p1,
                                                 static_cast<const T*>(x0m), static_cast<const T*>(x0L), smooth,
                                                 static_cast<T*>(means), static_cast<T*>(chols), scalars);
  }
  static const Ops* get() {
    static const Ops ops{&filter, &smoother, &smo_elements, &linearize, &scale_inplace, &sequential};
    return &ops;
  }
};

// One specialization per compiled shape (pof_inst_D<D>_d<d>.cu).
template <int D, int DY>
const Ops* ops_shape(int dtype);

// Runtime dispatch over the compiled shapes (pof_registry.cu); nullptr when
// the (dtype, D, d) combination is not compiled.
const Ops* find_shape(int dtype, int D, int DY);

}  // namespace pof
