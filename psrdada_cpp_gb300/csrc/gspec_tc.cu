// Tables and kernels of the tensor-core (split-precision) DFT-1024.
#include <cuda_runtime.h>

#include <cstdio>
#include <string>

#include "../../include/gspec.h"
#include "gspec_tc.cuh"
#include "gspec_tc_kernels.cuh"

namespace gspec {
namespace tc {

// DFT-32 operand of one stage as a logical [n][k] 64 x 64 matrix with
// n = 2c + s (output c, s = re/im) and k = 2a + r (input a, r = re/im):
//   Yr = sum xr cos + xi sin,  Yi = sum -xr sin + xi cos,  angle 2 pi a c / 32,
// split into hi + lo halves (BF16 or FP16 bit patterns) from FP64 values;
// and the 1024 twiddles W1024^j = exp(-2 pi i j / 1024) in FP32 from FP64.
__global__ void tables_kernel(uint16_t* hi, uint16_t* lo, float2* w1024, int bf16) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 64 * 64; i += gridDim.x * blockDim.x) {
    const int n = i >> 6, k = i & 63;
    const int c = n >> 1, s = n & 1, a = k >> 1, r = k & 1;
    double sn, cs;
    sincospi(2.0 * ((a * c) & 31) / 32.0, &sn, &cs);
    const double v = (s == 0) ? (r == 0 ? cs : sn) : (r == 0 ? -sn : cs);
    if (bf16) {
      const __nv_bfloat16 h = __double2bfloat16(v);
      const __nv_bfloat16 l = __double2bfloat16(v - static_cast<double>(__bfloat162float(h)));
      hi[i] = *reinterpret_cast<const uint16_t*>(&h);
      lo[i] = *reinterpret_cast<const uint16_t*>(&l);
    } else {
      const __half h = __double2half(v);
      const __half l = __double2half(v - static_cast<double>(__half2float(h)));
      hi[i] = *reinterpret_cast<const uint16_t*>(&h);
      lo[i] = *reinterpret_cast<const uint16_t*>(&l);
    }
  }
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < 1024; j += gridDim.x * blockDim.x) {
    double sn, cs;
    sincospi(2.0 * j / 1024.0, &sn, &cs);
    w1024[j] = make_float2(static_cast<float>(cs), static_cast<float>(-sn));
  }
}

cudaError_t launch_tables(uint16_t* hi, uint16_t* lo, float2* w1024, bool bf16, cudaStream_t s) {
  tables_kernel<<<16, 256, 0, s>>>(hi, lo, w1024, bf16 ? 1 : 0);
  return cudaGetLastError();
}

// Test kernel: ntiles x 4 transforms of 1024 points, global in/out.
template <bool BF16>
__global__ void __launch_bounds__(128) dft1024_test_kernel(const float2* __restrict__ in, float2* __restrict__ out,
                                                           const uint16_t* __restrict__ g_hi,
                                                           const uint16_t* __restrict__ g_lo,
                                                           const float2* __restrict__ g_w, uint32_t* err) {
  extern __shared__ __align__(1024) char smem[];
  TileSmem s;
  s.a_hi = smem;
  s.a_lo = smem + kABytes;
  s.b_hi = smem + 2 * kABytes;
  s.b_lo = smem + 2 * kABytes + kBBytes;
  float2* w = reinterpret_cast<float2*>(smem + 2 * kABytes + 2 * kBBytes);
  float2* xs = w + 1024;                                         // 4 x 1024 inputs, then outputs
  uint64_t* bar = reinterpret_cast<uint64_t*>(xs + 4 * 1024);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
  s.w = w;
  s.bar = bar;
  const int tid = threadIdx.x;
  load_dft32_operand(s.b_hi, s.b_lo, g_hi, g_lo, tid, 128);
  for (int i = tid; i < 1024; i += 128) w[i] = g_w[i];
  const float2* src = in + static_cast<size_t>(blockIdx.x) * 4 * 1024;
  for (int i = tid; i < 4 * 1024; i += 128) xs[i] = src[i];
  if (tid == 0) {
    mbar_init(bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  // 4x the accumulator columns: headroom for the test of the instruction encodings
  constexpr uint32_t kCols = 4 * kTmemCols;
  if (tid < 32) tmem_alloc(tmem_slot, kCols);
  fence_before();
  __syncthreads();
  fence_after();
  s.tmem = *tmem_slot;
  uint32_t phase = 0;
  const bool ok = dft1024_tile<BF16>(
      s, phase, tid, [&](int t, int n) { return xs[t * 1024 + n]; },
      [&](int t, int k, float2 v) { out[(static_cast<size_t>(blockIdx.x) * 4 + t) * 1024 + k] = v; });
  if (!ok && err) atomicExch(err, 3u);
  __syncthreads();
  fence_after();
  if (tid < 32) tmem_dealloc(s.tmem, kCols);
}

size_t test_smem_bytes() { return 2 * kABytes + 2 * kBBytes + 1024 * 8 + 4 * 1024 * 8 + 16; }

}  // namespace tc
}  // namespace gspec

using namespace gspec;

extern "C" int gspec_tc_dft1024_device(const void* d_in, void* d_out, uint32_t ntransforms, int form,
                                       void* cuda_stream) {
  if (!d_in || !d_out || ntransforms == 0 || ntransforms % 4) return GSPEC_ERR_ARG;
  if (form != GSPEC_FORM_BF16 && form != GSPEC_FORM_FP16) return GSPEC_ERR_ARG;
  const bool bf16 = form == GSPEC_FORM_BF16;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  uint16_t *hi = nullptr, *lo = nullptr;
  float2* w = nullptr;
  uint32_t* err = nullptr;
  int rc = GSPEC_OK;
  if (cudaMalloc(&hi, 4096 * 2) != cudaSuccess || cudaMalloc(&lo, 4096 * 2) != cudaSuccess ||
      cudaMalloc(&w, 1024 * sizeof(float2)) != cudaSuccess || cudaMalloc(&err, 4) != cudaSuccess) {
    rc = GSPEC_ERR_CUDA;
  } else {
    cudaMemsetAsync(err, 0, 4, s);
    tc::launch_tables(hi, lo, w, bf16, s);
    const size_t smem = tc::test_smem_bytes();
    auto kern = bf16 ? tc::dft1024_test_kernel<true> : tc::dft1024_test_kernel<false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    kern<<<ntransforms / 4, 128, smem, s>>>(static_cast<const float2*>(d_in), static_cast<float2*>(d_out), hi, lo, w,
                                             err);
    uint32_t h_err = 0;
    if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      rc = GSPEC_ERR_CUDA;
    else if (h_err)
      rc = GSPEC_ERR_CUDA;
  }
  cudaFree(hi);
  cudaFree(lo);
  cudaFree(w);
  cudaFree(err);
  return rc;
}
