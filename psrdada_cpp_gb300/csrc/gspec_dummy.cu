// Synthetic DADA blocks generated on the device: the producer side of the
// gated spectrometer's tests and benchmarks, replacing the reference's
// dummy_data_generator (psrdada_cpp/effelsberg/edd/src/dummy_data_generator.cu).
//
// Mode GSPEC_DUMMY_TWO_TONE restates that program's block: the real signal
// of a spectrum holding 50 at bin nFreqs/3 and 20 at bin nFreqs/2
// (nFreqs = n/2 + 1, n = the block's data samples; an unnormalised C2R, :130-137),
// i.e. x[t] = 100 cos(2 pi t k1 / n) + 40 cos(2 pi t k2 / n) (a bin at n/2
// is not doubled), rounded to float; quantised linearly between the
// block's own minimum and maximum to 0..255 (packNbit<8>, edd/Packer.cuh:32-41)
// and shifted to two's complement by -128 (:150-156).  The reference leaves
// the side-channel items unwritten; here they are zero.
//
// Mode GSPEC_DUMMY_STREAM writes the seeded stream the gated spectrometer's
// tests use: per pol, noise of standard deviation sigma (the sum of twelve
// 16-bit uniforms from a counter-based hash, centred: Irwin-Hall), plus a
// tone of tone_amplitude with tone_period samples per cycle, rounded and
// clipped to the bit depth, packed big-endian; the selected side-channel
// item of every heap carries the noise-diode state
// ((global heap / diode_period_heaps) & 1) in selected_bit and, for a
// lost_fraction of heaps (by the same hash), bit 63.  The block's position in
// the stream (block_index) continues the diode phase, the tone and the noise.
#include <cuda_runtime.h>

#include <cstdint>

#include "../../include/gspec.h"

namespace {

// splitmix64 finaliser: a counter-based hash of one 64-bit word
__host__ __device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

struct Geometry {
  uint64_t heap, nsc, nheaps, data_bytes, sc_off, samples_per_pol;
  uint32_t nbits, dual;
};

// byte address of pol-stream byte b (dual-pol heaps alternate P0 P1)
__device__ __forceinline__ uint64_t pol_addr(const Geometry& g, int pol, uint64_t b) {
  if (!g.dual) return b;
  const uint64_t h = b / g.heap;
  return (2 * h + pol) * g.heap + (b - h * g.heap);
}

// two's-complement sample value of sample s of pol `pol` in stream mode
__device__ __forceinline__ int stream_sample(const gspec_dummy_config& c, uint32_t nbits, int pol, uint64_t s) {
  const uint64_t key = mix64(c.seed ^ (0x51ED27ull * (pol + 1))) ^ s;
  const uint64_t h0 = mix64(key * 3), h1 = mix64(key * 3 + 1), h2 = mix64(key * 3 + 2);
  int64_t sum = 0;
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    sum += static_cast<int64_t>((h0 >> (16 * i)) & 0xFFFF);
    sum += static_cast<int64_t>((h1 >> (16 * i)) & 0xFFFF);
    sum += static_cast<int64_t>((h2 >> (16 * i)) & 0xFFFF);
  }
  // centred sum of 12 uniforms on [0, 65535]: standard deviation ~65536
  const double noise = static_cast<double>(sum - 393210) * static_cast<double>(c.sigma) / 65536.0;
  double tone = 0.0;
  if (c.tone_period > 0 && c.tone_amplitude != 0.f)
    tone = static_cast<double>(c.tone_amplitude) * cospi(2.0 * static_cast<double>(s % c.tone_period) /
                                                          static_cast<double>(c.tone_period));
  const double lo = -static_cast<double>(1 << (nbits - 1)), hi = static_cast<double>((1 << (nbits - 1)) - 1);
  return static_cast<int>(fmin(fmax(rint(noise + tone), lo), hi));
}

// packs group g (8 samples for 8 bit, 32 for 10 bit, 16 for 12 bit) of one
// pol: big-endian bit stream, MSB first
template <int NBITS>
__global__ void stream_samples_kernel(gspec_dummy_config c, Geometry g, uint8_t* block) {
  constexpr int GS = NBITS == 8 ? 8 : (NBITS == 10 ? 32 : 16);
  constexpr int GB = GS * NBITS / 8;
  const uint64_t groups = g.samples_per_pol / GS;
  const int npol = g.dual ? 2 : 1;
  for (uint64_t w = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; w < groups * npol;
       w += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const int pol = static_cast<int>(w % npol);
    const uint64_t grp = w / npol;
    uint8_t bytes[GB];
#pragma unroll
    for (int i = 0; i < GB; ++i) bytes[i] = 0;
#pragma unroll
    for (int i = 0; i < GS; ++i) {
      const uint64_t s = c.block_index * g.samples_per_pol + grp * GS + i;
      const uint32_t v = static_cast<uint32_t>(stream_sample(c, NBITS, pol, s)) & ((1u << NBITS) - 1);
      // bits [NBITS*i, NBITS*(i+1)) of the group, MSB first
#pragma unroll
      for (int b = 0; b < NBITS; ++b) {
        const int bit = NBITS * i + b;
        if ((v >> (NBITS - 1 - b)) & 1u) bytes[bit >> 3] |= static_cast<uint8_t>(0x80u >> (bit & 7));
      }
    }
    const uint64_t b0 = grp * GB;
#pragma unroll
    for (int i = 0; i < GB; ++i) block[pol_addr(g, pol, b0 + i)] = bytes[i];
  }
}

__global__ void stream_items_kernel(gspec_dummy_config c, Geometry g, uint8_t* block) {
  const uint64_t heaps_per_pol = g.dual ? g.nheaps / 2 : g.nheaps;
  const int npol = g.dual ? 2 : 1;
  uint64_t* items = reinterpret_cast<uint64_t*>(block + g.sc_off);
  for (uint64_t w = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; w < heaps_per_pol * npol * g.nsc;
       w += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint64_t item = w % g.nsc;
    const int pol = static_cast<int>((w / g.nsc) % npol);
    const uint64_t h = w / (g.nsc * npol);
    uint64_t v = 0;
    if (item == c.selected_side_channel) {
      const uint64_t gh = c.block_index * heaps_per_pol + h;
      if (c.diode_period_heaps) v |= ((gh / c.diode_period_heaps) & 1ull) << c.selected_bit;
      if (c.lost_fraction > 0.f) {
        const double u = static_cast<double>(mix64(c.seed ^ 0x10575EEDull ^ (gh * 2 + pol)) >> 11) * 0x1p-53;
        if (u < static_cast<double>(c.lost_fraction)) v |= 1ull << 63;
      }
    }
    // dual pol: items alternate P0 P1 item by item (pitch 16 B, edd/src/GatedSpectrometer.cu:285-300)
    items[(h * g.nsc + item) * npol + pol] = v;
  }
}

// two-tone signal of the reference generator, rounded to float
__device__ __forceinline__ float two_tone(uint64_t t, uint64_t n) {
  const uint64_t nfreq = n / 2 + 1;
  const uint64_t k1 = nfreq / 3, k2 = nfreq / 2;
  auto term = [&](uint64_t k, double amp) {
    const double w = (k == 0 || 2 * k == n) ? amp : 2.0 * amp;
    return w * cospi(2.0 * static_cast<double>((k * t) % n) / static_cast<double>(n));
  };
  return static_cast<float>(term(k1, 50.0) + term(k2, 20.0));
}

// order-preserving unsigned key of a float (for min / max by integer atomics)
__device__ __forceinline__ uint32_t fkey(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float fval(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// mm[0] = key of the minimum, mm[1] = key of the maximum (exact, order-free)
__global__ void two_tone_minmax_kernel(uint64_t n, uint32_t* mm) {
  uint32_t lo = 0xFFFFFFFFu, hi = 0u;
  for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const uint32_t k = fkey(two_tone(t, n));
    lo = min(lo, k);
    hi = max(hi, k);
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  if ((threadIdx.x & 31) == 0) {
    atomicMin(mm, lo);
    atomicMax(mm + 1, hi);
  }
}

__global__ void two_tone_pack_kernel(uint64_t n, const uint32_t* mm, uint8_t* block) {
  const float lo = fval(mm[0]), hi = fval(mm[1]);
  const float level = __fdiv_rn(__fsub_rn(hi, lo), 255.f);
  for (uint64_t t = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    float v = __fdiv_rn(__fsub_rn(two_tone(t, n), lo), level);
    v = fmaxf(fminf(v, 255.f), 0.f);
    block[t] = static_cast<uint8_t>(static_cast<int>(static_cast<uint32_t>(v)) - 128);
  }
}

}  // namespace

extern "C" int gspec_dummy_block_device(const gspec_dummy_config* c, void* d_block, void* d_work, void* cuda_stream) {
  if (!c || !d_block) return GSPEC_ERR_ARG;
  if (c->nbits != 8 && c->nbits != 10 && c->nbits != 12) return GSPEC_ERR_ARG;
  Geometry g{};
  g.heap = c->heap_size;
  g.nsc = c->n_side_channels;
  if (g.heap == 0) return GSPEC_ERR_ARG;
  g.nheaps = c->buffer_size / (g.heap + 8 * g.nsc);
  if (g.nheaps == 0 || (c->dual_pol && g.nheaps % 2)) return GSPEC_ERR_ARG;
  g.data_bytes = g.nheaps * g.heap;
  g.sc_off = c->buffer_size - 8 * g.nsc * g.nheaps;   // after the gap, as DadaBufferLayout places the items
  g.dual = c->dual_pol ? 1u : 0u;
  g.nbits = c->nbits;
  const uint64_t pol_bytes = g.dual ? g.data_bytes / 2 : g.data_bytes;
  g.samples_per_pol = pol_bytes * 8 / c->nbits;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  if (cudaMemsetAsync(d_block, 0, c->buffer_size, s) != cudaSuccess) return GSPEC_ERR_CUDA;
  if (c->mode == GSPEC_DUMMY_TWO_TONE) {
    // the reference's 8-bit block over the whole data region (no pols, no items)
    if (c->nbits != 8 || !d_work) return GSPEC_ERR_ARG;
    uint32_t* mm = static_cast<uint32_t*>(d_work);   // [min key, max key]
    if (cudaMemsetAsync(mm, 0xFF, 4, s) != cudaSuccess || cudaMemsetAsync(mm + 1, 0, 4, s) != cudaSuccess)
      return GSPEC_ERR_CUDA;
    two_tone_minmax_kernel<<<304, 256, 0, s>>>(g.data_bytes, mm);
    two_tone_pack_kernel<<<1216, 256, 0, s>>>(g.data_bytes, mm, static_cast<uint8_t*>(d_block));
    return cudaGetLastError() == cudaSuccess ? GSPEC_OK : GSPEC_ERR_CUDA;
  }
  if (c->mode != GSPEC_DUMMY_STREAM) return GSPEC_ERR_ARG;
  if (c->selected_side_channel >= g.nsc && g.nsc) return GSPEC_ERR_ARG;
  const int gsmp = c->nbits == 8 ? 8 : (c->nbits == 10 ? 32 : 16);
  if (g.samples_per_pol % gsmp || (g.dual && g.heap % (gsmp * c->nbits / 8))) return GSPEC_ERR_ARG;
  uint8_t* blk = static_cast<uint8_t*>(d_block);
  switch (c->nbits) {
    case 8: stream_samples_kernel<8><<<1216, 256, 0, s>>>(*c, g, blk); break;
    case 10: stream_samples_kernel<10><<<1216, 256, 0, s>>>(*c, g, blk); break;
    default: stream_samples_kernel<12><<<1216, 256, 0, s>>>(*c, g, blk); break;
  }
  if (g.nsc) stream_items_kernel<<<152, 256, 0, s>>>(*c, g, blk);
  return cudaGetLastError() == cudaSuccess ? GSPEC_OK : GSPEC_ERR_CUDA;
}

extern "C" int gspec_dummy_block(const gspec_dummy_config* c, void* host_block) {
  if (!c || !host_block) return GSPEC_ERR_ARG;
  void* d_block = nullptr;
  void* d_work = nullptr;
  int rc = GSPEC_ERR_CUDA;
  cudaStream_t s = nullptr;
  if (cudaMalloc(&d_block, c->buffer_size) == cudaSuccess && cudaMalloc(&d_work, 16) == cudaSuccess &&
      cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) == cudaSuccess) {
    rc = gspec_dummy_block_device(c, d_block, d_work, s);
    if (rc == GSPEC_OK && (cudaMemcpyAsync(host_block, d_block, c->buffer_size, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
                           cudaStreamSynchronize(s) != cudaSuccess))
      rc = GSPEC_ERR_CUDA;
  }
  if (s) cudaStreamDestroy(s);
  cudaFree(d_block);
  cudaFree(d_work);
  return rc;
}
