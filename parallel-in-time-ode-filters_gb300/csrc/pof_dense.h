// Entry points of the dense (large-D) filter/smoother, pof_dense.cu.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace pof {
namespace dense {

// The dense path takes every shape with D >= kMinD that the small-D tables
// do not compile.
constexpr int kMinD = 32;

// which: 0 filter, 1 filter + smoother, 2 smoother (x0m / x0L are then the
// filtered means / chols).  chunks: the number of chunks P (0: default).
size_t workspace_bytes(int dtype, int which, int64_t n, int D, int d, int chunks);
int filtsmooth(int which, int dtype, int64_t n, int D, int d, const void* x0m, const void* x0L, const void* F,
               const void* QL, int64_t fts, const void* H, const void* c, const void* R, int64_t rst, void* om,
               void* oL, double* osc, int chunks, void* ws, size_t wsb, cudaStream_t st);

// EK1 linearization (H, c) of a field the dense path linearizes
// (FIELD_FHN_RD) at means[1:]; p0, p1 the Nordsieck scales of E0, E1.
int linearize(int dtype, int64_t n, int D, int d, int field, const void* params, double p0, double p1,
              const void* means, void* H, void* c, cudaStream_t st);

}  // namespace dense
}  // namespace pof
