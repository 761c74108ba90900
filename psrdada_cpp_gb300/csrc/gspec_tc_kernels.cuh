// Launchers of the tensor-core (split-precision) four-step form.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "gspec_kernels.cuh"

namespace gspec {
namespace tc {
// DFT-32 operand halves ([n][k] 64 x 64, 16-bit patterns) and W1024 twiddles from FP64.
cudaError_t launch_tables(uint16_t* hi, uint16_t* lo, float2* w1024, bool bf16, cudaStream_t s);
// Pass A (pass 0, needs N1 = 1024) or pass B (pass 1, needs N2 = 1024) on the tensor cores.
cudaError_t launch_tc_pass(int pass, int nbits, bool dual, const FourStepParams& p, cudaStream_t s);
}  // namespace tc
}  // namespace gspec
