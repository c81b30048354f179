// Opt-in per-kernel timing: CUDA events recorded on the launching stream
// around every libpof launch, summed per kernel kind when collected.
// Off by default (no events recorded, no overhead).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace pof {

enum ProfKind : int {
  PK_LINEARIZE = 0,
  PK_FILT_L0_REDUCE,
  PK_FILT_REDUCE,
  PK_FILT_TOP,
  PK_FILT_DOWN,
  PK_FILT_L0_DOWN,
  PK_FILT_FINALIZE,
  PK_SMO_L0_REDUCE,
  PK_SMO_REDUCE,
  PK_SMO_TOP,
  PK_SMO_DOWN,
  PK_SMO_L0_DOWN,
  PK_SMO_FINALIZE,
  PK_CONTROL,
  PK_SEQUENTIAL,
  PK_COUNT
};

bool prof_on();
void prof_begin(int kind, cudaStream_t st);
void prof_end(int kind, cudaStream_t st);
void prof_flush();  // sum the finished event pairs (waits for them)

// Status helpers shared by the C-ABI translation units (pof_capi.cu).
int cuda_status(cudaError_t e);
int launch_status();
char* aligned_ws(void* ws);  // first 256-byte boundary at or after ws

}  // namespace pof
