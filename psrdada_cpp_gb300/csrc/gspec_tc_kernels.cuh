// Launchers of the tensor-core (split-precision) four-step form.
#pragma once

#include <cuda_runtime.h>
#include <cstdint>

#include "gspec_kernels.cuh"

namespace gspec {
namespace tc {
constexpr uint64_t kImageBytesHost = 3 * 9216 + 1024 * 8;   // kImageBytes of gspec_tc.cuh
constexpr uint64_t kTableParts = 3;                          // kMaxParts of gspec_tc.cuh
// DFT-32 operand parts (kTableParts x [n][k] 64 x 64, 16-bit patterns) and W1024 twiddles from FP64.
cudaError_t launch_tables(uint16_t* parts, float2* w1024, bool bf16, cudaStream_t s);
// Shared-memory image [B1 | B2 | B3 | W1024] (35840 bytes) from the tables.
cudaError_t launch_image(const uint16_t* parts, const float2* w, uint8_t* img, cudaStream_t s);
// Pass A (pass 0, needs N1 = 1024) or pass B (pass 1, needs N2 = 1024) on the tensor cores.
cudaError_t launch_tc_pass(int pass, int nbits, bool dual, const FourStepParams& p, cudaStream_t s);
}  // namespace tc
}  // namespace gspec
