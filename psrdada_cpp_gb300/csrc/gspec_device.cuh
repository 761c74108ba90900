// Device building blocks of the gated spectrometer (sm_103a).
//
//  * bit-stream unpack of big-endian two's-complement 8/10/12-bit samples
//    (the arithmetic of edd/src/Unpacker.cu:24-108 and
//    edd/test/src/UnpackerTester.cu:41-201, written as funnel shifts over
//    byte-swapped 32-bit words);
//  * the side-channel gate (edd/src/GatedSpectrometer.cu:22-59) with the
//    reference's exact float formula (v - b) * m + b;
//  * register DFTs of radix 2/4/8/16 and a shared-memory Stockham FFT used
//    by every FFT kernel of the library (replaces cuFFT R2C,
//    edd/detail/GatedSpectrometer.cu:144-145,281-288).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace gspec {

// ---------------------------------------------------------------- complex
struct __align__(8) cf { float x, y; };

#ifndef GSPEC_F32X2
#define GSPEC_F32X2 1
#endif
#if GSPEC_F32X2
// Complex add and subtract as one packed two-lane FP32 instruction each
// (add/sub.rn.f32x2, sm_100 and later) on the float2 held as a 64-bit pair.
__device__ __forceinline__ unsigned long long f2_pack(float2 a) {
  unsigned long long r;
  asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(a.x), "f"(a.y));
  return r;
}
__device__ __forceinline__ float2 f2_unpack(unsigned long long r) {
  float2 a;
  asm("mov.b64 {%0, %1}, %2;" : "=f"(a.x), "=f"(a.y) : "l"(r));
  return a;
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(d);
}
__device__ __forceinline__ float2 csub(float2 a, float2 b) {
  unsigned long long d;
  asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_pack(a)), "l"(f2_pack(b)));
  return f2_unpack(d);
}
#else
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
#endif
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
// multiply by -i
__device__ __forceinline__ float2 cmul_mi(float2 a) { return make_float2(a.y, -a.x); }

// ------------------------------------------------------------ smem padding
// One float2 of padding per 16 keeps the Stockham stores (stride R) and the
// unpack stores (stride G) free of bank conflicts for R, G in {8, 16}.
__device__ __forceinline__ int spad(int i) { return i + (i >> 4); }
__host__ __device__ constexpr int spad_size(int n) { return n + (n >> 4); }

// ------------------------------------------------------------- register DFTs
// Forward DFT (W = exp(-2 pi i / R)), natural order in and out.
__device__ __forceinline__ void dft2(float2& a, float2& b) {
  float2 t = a;
  a = cadd(t, b);
  b = csub(t, b);
}

__device__ __forceinline__ void dft4(float2& v0, float2& v1, float2& v2, float2& v3) {
  float2 t0 = cadd(v0, v2), t1 = csub(v0, v2);
  float2 t2 = cadd(v1, v3), t3 = cmul_mi(csub(v1, v3));
  v0 = cadd(t0, t2);
  v2 = csub(t0, t2);
  v1 = cadd(t1, t3);
  v3 = csub(t1, t3);
}

constexpr float kS2 = 0.70710678118654752f;   // sqrt(1/2)
constexpr float kC8 = 0.92387953251128674f;   // cos(pi/8)
constexpr float kS8 = 0.38268343236508977f;   // sin(pi/8)

// multiply by W8^1 = (1 - i)/sqrt2
__device__ __forceinline__ float2 w8_1(float2 a) { return make_float2(kS2 * (a.x + a.y), kS2 * (a.y - a.x)); }
// multiply by W8^3 = (-1 - i)/sqrt2
__device__ __forceinline__ float2 w8_3(float2 a) { return make_float2(kS2 * (a.y - a.x), -kS2 * (a.x + a.y)); }
// multiply by W16^1 = cos(pi/8) - i sin(pi/8)
__device__ __forceinline__ float2 w16_1(float2 a) {
  return make_float2(fmaf(a.x, kC8, a.y * kS8), fmaf(a.y, kC8, -a.x * kS8));
}
// multiply by W16^3 = sin(pi/8) - i cos(pi/8)
__device__ __forceinline__ float2 w16_3(float2 a) {
  return make_float2(fmaf(a.x, kS8, a.y * kC8), fmaf(a.y, kS8, -a.x * kC8));
}
// multiply by W16^9 = -W16^1
__device__ __forceinline__ float2 w16_9(float2 a) {
  return make_float2(-fmaf(a.x, kC8, a.y * kS8), -fmaf(a.y, kC8, -a.x * kS8));
}

__device__ __forceinline__ void dft8(float2 (&v)[8]) {
  // 8 = 2 x 4: v[a + 2b], a in {0,1}, b in 0..3
  dft4(v[0], v[2], v[4], v[6]);
  dft4(v[1], v[3], v[5], v[7]);
  // y[a][c] lives in v[a + 2c]; twiddle W8^(a*c)
  v[3] = w8_1(v[3]);
  v[5] = cmul_mi(v[5]);
  v[7] = w8_3(v[7]);
  // V[c + 4d] = y0[c] + W2^d y1[c]
  float2 o[8];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    o[c] = cadd(v[2 * c], v[2 * c + 1]);
    o[c + 4] = csub(v[2 * c], v[2 * c + 1]);
  }
#pragma unroll
  for (int i = 0; i < 8; ++i) v[i] = o[i];
}

__device__ __forceinline__ void dft16(float2 (&v)[16]) {
  // 16 = 4 x 4: v[a + 4b]; stage 1 DFT4 over b for each a
#pragma unroll
  for (int a = 0; a < 4; ++a) dft4(v[a], v[a + 4], v[a + 8], v[a + 12]);
  // y[a][c] in v[a + 4c]; twiddle W16^(a*c)
  v[5] = w16_1(v[5]);                 // a1 c1
  v[9] = w8_1(v[9]);                  // a1 c2 : W16^2
  v[13] = w16_3(v[13]);               // a1 c3
  v[6] = w8_1(v[6]);                  // a2 c1 : W16^2
  v[10] = cmul_mi(v[10]);             // a2 c2 : W16^4
  v[14] = w8_3(v[14]);                // a2 c3 : W16^6
  v[7] = w16_3(v[7]);                 // a3 c1
  v[11] = w8_3(v[11]);                // a3 c2 : W16^6
  v[15] = w16_9(v[15]);               // a3 c3
  // stage 2: DFT4 over a for each c; V[c + 4d]
  float2 o[16];
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    float2 y0 = v[4 * c], y1 = v[4 * c + 1], y2 = v[4 * c + 2], y3 = v[4 * c + 3];
    dft4(y0, y1, y2, y3);
    o[c] = y0;
    o[c + 4] = y1;
    o[c + 8] = y2;
    o[c + 12] = y3;
  }
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = o[i];
}

template <int R>
__device__ __forceinline__ void dft(float2 (&v)[R]) {
  if constexpr (R == 2) {
    dft2(v[0], v[1]);
  } else if constexpr (R == 4) {
    dft4(v[0], v[1], v[2], v[3]);
  } else if constexpr (R == 8) {
    dft8(v);
  } else {
    static_assert(R == 16, "radix");
    dft16(v);
  }
}

// ------------------------------------------------------ Stockham FFT plan
// N = 16^a * r, r in {1,2,4,8}: passes of radix 16 then one of radix r.
__host__ __device__ constexpr int ilog2c(int n) { return n <= 1 ? 0 : 1 + ilog2c(n / 2); }
__host__ __device__ constexpr int pass_radix(int n, int ns) { return (n / ns) >= 16 ? 16 : (n / ns); }
// offset (in float2) of the twiddle table of the pass whose span is ns
__host__ __device__ constexpr int tw_offset(int n, int ns) {
  int off = 0;
  for (int s = 1; s < ns; s *= pass_radix(n, s)) {
    if (s > 1) off += s * pass_radix(n, s);
  }
  return off;
}
__host__ __device__ constexpr int tw_size(int n) { return tw_offset(n, n); }

// Barrier of a group of threads that share data: the whole CTA
// (kSyncCta), the calling warp (kSyncWarp: the group lies within one warp,
// every thread of the warp calls it) or the named barrier `id` of `count`
// threads (kSyncNamed: whole warps, ids 1..15; id 0 is __syncthreads').
constexpr int kSyncCta = 0, kSyncWarp = 1, kSyncNamed = 2;
template <int SYNC>
__device__ __forceinline__ void group_sync(int id, int count) {
  if constexpr (SYNC == kSyncWarp) {
    __syncwarp();
  } else if constexpr (SYNC == kSyncNamed) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
  } else {
    __syncthreads();
  }
}

// One in-place FFT of N points in padded shared memory S, done by the
// T = N/P threads with index t of the calling group.  Every thread of the
// group's barrier (group_sync<SYNC>: the CTA by default) must call it the
// same number of times.
// tw: per-pass tables, entry [k][q] = exp(-2 pi i q k / (ns R)) at
// tw_offset(N, ns) + k*ns + q; the kernels keep a copy in shared memory
// (load_twiddles) so the passes do not wait on global loads.
template <int N, int P, int NS = 1, int SYNC = kSyncCta>
__device__ __forceinline__ void fft_smem(float2* S, const float2* tw, int t, bool active, int bar_id = 0) {
  static_assert(SYNC != kSyncWarp || N / P <= 32, "a warp-synchronous FFT lies within one warp");
  auto sync = [&] { group_sync<SYNC>(bar_id, N / P); };
  if constexpr (NS < N) {
    constexpr int R = pass_radix(N, NS);
    constexpr int T = N / P;
    constexpr int NB = P / R;
    static_assert(P % R == 0, "points per thread must be a multiple of the radix");
    float2 v[NB][R];
    if (active) {
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        const int j = t + T * u;
#pragma unroll
        for (int k = 0; k < R; ++k) v[u][k] = S[spad(j + k * (N / R))];
      }
    }
    sync();
    if (active) {
#pragma unroll
      for (int u = 0; u < NB; ++u) {
        const int j = t + T * u;
        const int q = j & (NS - 1);
        if constexpr (NS > 1) {
          constexpr int TO = tw_offset(N, NS);
#pragma unroll
          for (int k = 1; k < R; ++k) v[u][k] = cmul(v[u][k], tw[TO + k * NS + q]);
        }
        dft<R>(v[u]);
        const int base = (j - q) * R + q;
#pragma unroll
        for (int k = 0; k < R; ++k) S[spad(base + k * NS)] = v[u][k];
      }
    }
    sync();
    fft_smem<N, P, NS * R, SYNC>(S, tw, t, active, bar_id);
  }
}

// The same FFT when the input sits unpadded in `src` (a TMA staging buffer):
// the first pass (span 1, no twiddles) reads src and writes S (padded); the
// remaining passes run in S.  The caller makes src valid for all threads
// before the call (mbarrier wait) and S free of readers.
template <int N, int P>
__device__ __forceinline__ void fft_smem_from(const float2* src, float2* S, const float2* tw, int t, bool active) {
  constexpr int R = pass_radix(N, 1);
  constexpr int T = N / P;
  constexpr int NB = P / R;
  if (active) {
#pragma unroll
    for (int u = 0; u < NB; ++u) {
      const int j = t + T * u;
      float2 v[R];
#pragma unroll
      for (int k = 0; k < R; ++k) v[k] = src[j + k * (N / R)];
      dft<R>(v);
#pragma unroll
      for (int k = 0; k < R; ++k) S[spad(j * R + k)] = v[k];
    }
  }
  __syncthreads();
  fft_smem<N, P, R>(S, tw, t, active);
}

// Copies the Stockham tables of an N-point FFT (tw_size(N) entries) from
// global to shared memory; the caller synchronises before use.
template <int N>
__device__ __forceinline__ void load_twiddles(float2* dst, const float2* __restrict__ src) {
  constexpr int n = tw_size(N);
  for (int i = threadIdx.x; i < n; i += blockDim.x) dst[i] = __ldg(src + i);
}

// ------------------------------------------------------- TMA bulk copies
// One-dimensional bulk copies global -> shared completing on an mbarrier
// (sm_90+ cp.async.bulk).  Addresses and sizes must be multiples of 16 B.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}
// Waits for the given phase parity; gives up after `limit` polls and
// returns false (the caller records an error instead of hanging).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
  const uint32_t a = smem_addr(bar);
  for (uint32_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// ------------------------------------------------------------------ unpack
// A group is the smallest whole number of samples that starts on a 64-bit
// word: 8 samples / 8 bytes (8 bit), 32 / 40 (10 bit), 16 / 24 (12 bit).
template <int NBITS> struct Group;
template <> struct Group<8> { static constexpr int samples = 8, words = 1; };
template <> struct Group<10> { static constexpr int samples = 32, words = 5; };
template <> struct Group<12> { static constexpr int samples = 16, words = 3; };

__device__ __forceinline__ uint32_t bswap32(uint32_t x) { return __byte_perm(x, 0, 0x0123); }

// Unpack one group from `p` (8-byte aligned, global memory) into out[]
// as signed integers.  The 64-bit words are read as little-endian 32-bit
// halves and byte-swapped into a big-endian bit stream W[0..2*words).
// 12-bit groups (three words) are read as one 16-byte load on the 16-byte
// aligned side and one 8-byte load.
#ifndef GSPEC_GROUP_WIDE
#define GSPEC_GROUP_WIDE 1
#endif
template <int NBITS>
__device__ __forceinline__ void unpack_group(const uint8_t* __restrict__ p, int (&out)[Group<NBITS>::samples]) {
  constexpr int NG = Group<NBITS>::words;
  constexpr int NW = 2 * NG;
  uint32_t W[NW + 1];
  const uint2* q = reinterpret_cast<const uint2*>(p);
  uint2 u[NG];
  if constexpr (NG != 3 || !GSPEC_GROUP_WIDE) {
    // one word (8 bit); five (10 bit) stay 8-byte loads: the 16-byte form
    // costs the 10-bit column pass registers
#pragma unroll
    for (int w = 0; w < NG; ++w) u[w] = __ldg(q + w);
  } else if (reinterpret_cast<uintptr_t>(p) & 8u) {
    // one word before the 16-byte boundary, then pairs
    u[0] = __ldg(q);
#pragma unroll
    for (int a = 1; a + 1 < NG; a += 2) {
      const uint4 t = __ldg(reinterpret_cast<const uint4*>(q + a));
      u[a] = make_uint2(t.x, t.y);
      u[a + 1] = make_uint2(t.z, t.w);
    }
    if constexpr ((NG & 1) == 0) u[NG - 1] = __ldg(q + NG - 1);
  } else {
    // pairs from p on, then a last word when NG is odd
#pragma unroll
    for (int a = 0; a + 1 < NG; a += 2) {
      const uint4 t = __ldg(reinterpret_cast<const uint4*>(q + a));
      u[a] = make_uint2(t.x, t.y);
      u[a + 1] = make_uint2(t.z, t.w);
    }
    if constexpr (NG & 1) u[NG - 1] = __ldg(q + NG - 1);
  }
#pragma unroll
  for (int w = 0; w < NG; ++w) {
    W[2 * w] = bswap32(u[w].x);
    W[2 * w + 1] = bswap32(u[w].y);
  }
  W[NW] = 0;
#pragma unroll
  for (int i = 0; i < Group<NBITS>::samples; ++i) {
    constexpr int dummy = 0;
    (void)dummy;
    const int bit = NBITS * i;
    const int w = bit >> 5, sh = bit & 31;
    // bits [sh, sh+32) of W[w]:W[w+1] (MSB first)
    const uint32_t win = __funnelshift_l(W[w + 1], W[w], sh);
    out[i] = static_cast<int32_t>(win) >> (32 - NBITS);
  }
}

// Unpack S samples that start on a 4-byte boundary (S * NBITS a multiple of
// 32 bits): the part of a group that a tile narrower than the group keeps.
#ifndef GSPEC_SPAN_WIDE
#define GSPEC_SPAN_WIDE 1
#endif
// win16: p lies in a buffer made of whole 16-byte chunks, so the aligned
// 16-byte chunk around the span may be read whole.
template <int NBITS, int S>
__device__ __forceinline__ void unpack_span(const uint8_t* __restrict__ p, int (&out)[S], bool win16 = false) {
  if constexpr (S == Group<NBITS>::samples) {
    unpack_group<NBITS>(p, out);
  } else {
    static_assert((S * NBITS) % 32 == 0, "a span is whole 32-bit words");
    constexpr int NW = S * NBITS / 32;
    uint32_t W[NW + 1];
    const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
    if constexpr (NW == 3 && GSPEC_SPAN_WIDE) {
      // three words: one 16-byte load when they lie in one aligned 16-byte
      // chunk of a whole-chunk buffer, else one 8-byte and one 4-byte load
      // (the 8-byte one on whichever side of p is 8-byte aligned)
      const uint32_t mis = static_cast<uint32_t>(reinterpret_cast<uintptr_t>(p) & 15u);
      if (win16 && mis <= 4u) {
        const uint4 t = __ldg(reinterpret_cast<const uint4*>(p - mis));
        W[0] = bswap32(mis ? t.y : t.x);
        W[1] = bswap32(mis ? t.z : t.y);
        W[2] = bswap32(mis ? t.w : t.z);
      } else if (mis & 4u) {
        const uint2 t = __ldg(reinterpret_cast<const uint2*>(q + 1));
        W[0] = bswap32(__ldg(q));
        W[1] = bswap32(t.x);
        W[2] = bswap32(t.y);
      } else {
        const uint2 t = __ldg(reinterpret_cast<const uint2*>(q));
        W[0] = bswap32(t.x);
        W[1] = bswap32(t.y);
        W[2] = bswap32(__ldg(q + 2));
      }
    } else if constexpr (NW % 4 == 0) {
      if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0) {
#pragma unroll
        for (int w = 0; w < NW; w += 4) {
          const uint4 t = __ldg(reinterpret_cast<const uint4*>(q + w));
          W[w] = bswap32(t.x);
          W[w + 1] = bswap32(t.y);
          W[w + 2] = bswap32(t.z);
          W[w + 3] = bswap32(t.w);
        }
      } else {
#pragma unroll
        for (int w = 0; w < NW; ++w) W[w] = bswap32(__ldg(q + w));
      }
    } else {
#pragma unroll
      for (int w = 0; w < NW; ++w) W[w] = bswap32(__ldg(q + w));
    }
    W[NW] = 0;
#pragma unroll
    for (int i = 0; i < S; ++i) {
      const int bit = NBITS * i;
      const int w = bit >> 5, sh = bit & 31;
      const uint32_t win = __funnelshift_l(W[w + 1], W[w], sh);
      out[i] = static_cast<int32_t>(win) >> (32 - NBITS);
    }
  }
}

// ---------------------------------------------------------------- gating
// Side-channel gate of one sample (edd/src/GatedSpectrometer.cu:49-52):
//   G1 = (v - b1) * bit * !lost + b1 ;  G0 = (v - b0) * !bit * !lost + b0
// evaluated with explicit round-to-nearest float ops so no contraction or
// fast-math rewrite changes a bit of the result.
__device__ __forceinline__ float gate_value(float v, float b, bool m) {
  return m ? __fadd_rn(__fsub_rn(v, b), b) : b;
}

// Gate parameters shared by all kernels.
struct GateParams {
  const uint8_t* block;      // device copy of the whole DADA block
  uint64_t sc_offset;        // byte offset of the side-channel items
  uint32_t heap_size;        // bytes per heap
  uint32_t nsc;              // items per heap
  uint32_t sel;              // selected item
  uint32_t bitpos;           // selected bit
  uint32_t dual;             // 1: heaps and items alternate P0 P1
  uint32_t convention;       // 0 intended, 1 reference
  // intended: item = ((s * nbits) / (8 * heap_size)) * nsc + sel
  // reference: item = (s / chunk) * step + ((s % chunk) / heap_size) * nsc + sel
  uint32_t chunk;            // samples per gating chunk (reference)
  uint32_t step;             // items per gating chunk (reference)
  uint32_t nbits;
  int32_t heap_shift;        // intended convention: log2(samples per heap) when that is an integer power of 2, else -1
  const uint8_t* masks;      // per item index: bit0 = gate 0 (m0), bit1 = gate 1 (m1); built by the mask pass
  uint64_t heap_magic;       // ceil(2^64 / heap_size), 0 for heap_size 1 (see heap_of)
  uint32_t win16;            // 1: the block is 16-byte aligned and a whole number of 16-byte chunks long
};

// n / heap_size for 32-bit n without a division: with M = ceil(2^64 / d) =
// 2^64/d + e (0 <= e < 1), n*M/2^64 = n/d + n*e/2^64 and n*e/2^64 < 2^-32 < 1/d,
// which never carries floor(n/d) past the next integer (d < 2^32).
__device__ __forceinline__ uint32_t heap_of(const GateParams& g, uint32_t n) {
  return g.heap_magic ? static_cast<uint32_t>(__umul64hi(n, g.heap_magic)) : n;
}

__device__ __forceinline__ uint32_t item_index(const GateParams& g, uint32_t s) {
  if (g.convention == 1) {
    const uint32_t j = s / g.chunk;
    const uint32_t t = s - j * g.chunk;
    return j * g.step + heap_of(g, t) * g.nsc + g.sel;
  }
  if (g.heap_shift >= 0) return (s >> g.heap_shift) * g.nsc + g.sel;
  const uint64_t bit = static_cast<uint64_t>(s) * g.nbits;
  return static_cast<uint32_t>(bit / (8ull * g.heap_size)) * g.nsc + g.sel;
}

// Byte address of pol-stream byte b (dual-pol heaps alternate P0 P1).
// (pol byte offsets are below 2^32, checked by the host, so heap_of applies)
__device__ __forceinline__ const uint8_t* pol_byte(const GateParams& g, int pol, uint64_t b) {
  if (!g.dual) return g.block + b;
  const uint32_t b32 = static_cast<uint32_t>(b);
  const uint32_t h = heap_of(g, b32);
  return g.block + (2ull * h + pol) * g.heap_size + (b32 - h * g.heap_size);
}

// L2 prefetch of the sector holding p (no register result, no wait).
__device__ __forceinline__ void prefetch_l2(const void* p) {
  asm volatile("prefetch.global.L2 [%0];" ::"l"(p));
}

// Selected item after the dual-pol merge (edd/src/GatedSpectrometer.cu:9-19:
// logical OR in the reference convention, bitwise OR in the intended one).
__device__ __forceinline__ uint64_t load_item(const GateParams& g, uint32_t idx) {
  const uint64_t* items = reinterpret_cast<const uint64_t*>(g.block + g.sc_offset);
  if (!g.dual) return __ldg(items + idx);
  const uint64_t a = __ldg(items + 2ull * idx);
  const uint64_t b = __ldg(items + 2ull * idx + 1);
  if (g.convention == 1) return (a != 0 || b != 0) ? 1ull : 0ull;
  return a | b;
}

// Gate masks of an item: m0 = bit clear and heap kept, m1 = bit set and kept.
__device__ __forceinline__ void item_masks(uint64_t item, uint32_t bitpos, bool& m0, bool& m1) {
  const bool bit = (item >> bitpos) & 1ull;
  const bool lost = (item >> 63) & 1ull;
  m0 = !bit && !lost;
  m1 = bit && !lost;
}

// Per-thread gate statistics.
struct GateStats {
  uint32_t n0 = 0, n1 = 0, sat0 = 0, sat1 = 0;
  long long s0 = 0, s1 = 0;
};

// Exact sum of one gated sequence's in-gate values (the four-step path's
// DC bins): s = sum of the integer samples, n = their count, r = the sum of
// the rounding residues (v - b) + b - v of the reference's gate formula.  A
// residue is the difference of a float and the integer sample (|v| <= 2048)
// it rounds to within one ulp, so it is a multiple of 2^-24 of at most 2^-12
// in magnitude: a thread's sum of at most 128 of them is exact in FP32.  The
// out-of-gate samples are the baseline; the reader adds (N - n) * b.
struct DcAcc {
  int s = 0, n = 0;
  float r = 0.f;
};

// Gate masks of an item index from the mask pass.
__device__ __forceinline__ void mask_of(const GateParams& g, uint32_t idx, bool& m0, bool& m1) {
  const uint32_t m = __ldg(g.masks + idx);
  m0 = m & 1u;
  m1 = (m >> 1) & 1u;
}

// Unpack + gate one group of samples of one pol starting at pol sample s.
// Writes gated G0/G1 floats into g0[], g1[]; adds the statistics of gate 0
// when (stat_gates & 1) and of gate 1 when (stat_gates & 2), so that a
// sample visited by two jobs is counted once.
template <int NBITS, int GS = Group<NBITS>::samples>
__device__ __forceinline__ void gate_group(const GateParams& g, int pol, uint32_t s, float b0, float b1,
                                           float (&g0)[GS], float (&g1)[GS],
                                           GateStats& st, uint32_t stat_gates = 3u, DcAcc* dc0 = nullptr,
                                           DcAcc* dc1 = nullptr) {
  int v[GS];
  const uint64_t byte0 = static_cast<uint64_t>(s) * NBITS / 8;
  unpack_span<NBITS, GS>(pol_byte(g, pol, byte0), v, g.win16 != 0);
  const uint32_t ia = item_index(g, s);
  const uint32_t ib = item_index(g, s + GS - 1);
  bool a0, a1;
  mask_of(g, ia, a0, a1);
  bool c0 = a0, c1 = a1;
  uint32_t boundary = 0xffffffffu;
  if (ib != ia) {
    mask_of(g, ib, c0, c1);
    // first sample whose item is ib
    boundary = s;
    while (boundary < s + GS && item_index(g, boundary) == ia) ++boundary;
  }
  const bool k0 = stat_gates & 1u, k1 = stat_gates & 2u;
  constexpr int lo = -(1 << (NBITS - 1)), hi = (1 << (NBITS - 1)) - 1;
  if (ib == ia) {
    // the whole group lies in one heap: statistics per group
    int sumv = 0, satc = 0;
    float r0 = 0.f, r1 = 0.f;
#pragma unroll
    for (int i = 0; i < GS; ++i) {
      const float vf = static_cast<float>(v[i]);
      g0[i] = gate_value(vf, b0, a0);
      g1[i] = gate_value(vf, b1, a1);
      if (dc0) {
        r0 += g0[i] - vf;
        r1 += g1[i] - vf;
      }
      sumv += v[i];
      satc += (v[i] == lo) | (v[i] == hi);
    }
    if (a0 && k0) {
      st.n0 += GS;
      st.s0 += sumv;
      st.sat0 += satc;
      if (dc0) {
        dc0->s += sumv;
        dc0->n += GS;
        dc0->r += r0;
      }
    }
    if (a1 && k1) {
      st.n1 += GS;
      st.s1 += sumv;
      st.sat1 += satc;
      if (dc1) {
        dc1->s += sumv;
        dc1->n += GS;
        dc1->r += r1;
      }
    }
    return;
  }
#pragma unroll
  for (int i = 0; i < GS; ++i) {
    const bool second = (s + i) >= boundary;
    const bool m0 = second ? c0 : a0;
    const bool m1 = second ? c1 : a1;
    const float vf = static_cast<float>(v[i]);
    g0[i] = gate_value(vf, b0, m0);
    g1[i] = gate_value(vf, b1, m1);
    const bool sat = (v[i] == lo) | (v[i] == hi);
    const bool q0 = m0 && k0, q1 = m1 && k1;
    st.n0 += q0;
    st.n1 += q1;
    st.sat0 += (q0 && sat);
    st.sat1 += (q1 && sat);
    st.s0 += q0 ? v[i] : 0;
    st.s1 += q1 ? v[i] : 0;
    if (dc0 && q0) {
      dc0->s += v[i];
      dc0->n += 1;
      dc0->r += g0[i] - vf;
    }
    if (dc1 && q1) {
      dc1->s += v[i];
      dc1->n += 1;
      dc1->r += g1[i] - vf;
    }
  }
}

#ifndef GSPEC_SIMD8
#define GSPEC_SIMD8 1
#endif

// One gate of one group: out[] = gate `gate` of the samples; statistics of
// that gate only when `stats` is set.  8-bit spans of whole 16-byte chunks
// keep the raw words: a sample is the sign-extended byte at its address, and
// a span inside one item sums its samples four at a time (dp4a against
// 0x01010101) and counts its saturated ones by byte compares (-128 = 0x80,
// 127 = 0x7f) and a population count.
template <int NBITS, int GS = Group<NBITS>::samples>
__device__ __forceinline__ void gate_group1(const GateParams& g, int pol, uint32_t s, float b, int gate,
                                            float (&out)[GS], GateStats& st, bool stats, DcAcc* dc = nullptr) {
  constexpr bool kSimd8 = GSPEC_SIMD8 && NBITS == 8 && GS % 16 == 0;
  int v[GS];
  const uint64_t byte0 = static_cast<uint64_t>(s) * NBITS / 8;
  [[maybe_unused]] uint32_t raw[kSimd8 ? GS / 4 : 1];
  if constexpr (kSimd8) {
    // the span starts on a 4-byte boundary (GS samples of whole words)
    const uint8_t* p = pol_byte(g, pol, byte0);
    const uint32_t* q = reinterpret_cast<const uint32_t*>(p);
    if ((reinterpret_cast<uintptr_t>(p) & 15u) == 0) {
#pragma unroll
      for (int w = 0; w < GS / 4; w += 4) {
        const uint4 t = __ldg(reinterpret_cast<const uint4*>(q + w));
        raw[w] = t.x;
        raw[w + 1] = t.y;
        raw[w + 2] = t.z;
        raw[w + 3] = t.w;
      }
    } else {
#pragma unroll
      for (int w = 0; w < GS / 4; ++w) raw[w] = __ldg(q + w);
    }
#pragma unroll
    for (int i = 0; i < GS; ++i) v[i] = static_cast<int>(static_cast<int8_t>(raw[i >> 2] >> (8 * (i & 3))));
  } else {
    unpack_span<NBITS, GS>(pol_byte(g, pol, byte0), v, g.win16 != 0);
  }
  const uint32_t ia = item_index(g, s);
  const uint32_t ib = item_index(g, s + GS - 1);
  const uint32_t sh = gate ? 1u : 0u;
  const bool ma = (__ldg(g.masks + ia) >> sh) & 1u;
  constexpr int lo = -(1 << (NBITS - 1)), hi = (1 << (NBITS - 1)) - 1;
  int sumv = 0, satc = 0, cnt = 0;
  float res = 0.f;
  if (ib == ia) {
#pragma unroll
    for (int i = 0; i < GS; ++i) {
      const float vf = static_cast<float>(v[i]);
      out[i] = gate_value(vf, b, ma);
      if (dc) res += out[i] - vf;
      if constexpr (!kSimd8) {
        sumv += v[i];
        satc += (v[i] == lo) | (v[i] == hi);
      }
    }
    if constexpr (kSimd8) {
      uint32_t satbits = 0;
#pragma unroll
      for (int w = 0; w < GS / 4; ++w) {
        sumv = __dp4a(static_cast<int>(raw[w]), 0x01010101, sumv);
        satbits += __popc(__vcmpeq4(raw[w], 0x80808080u) | __vcmpeq4(raw[w], 0x7f7f7f7fu));
      }
      satc = static_cast<int>(satbits >> 3);
    }
    cnt = ma ? GS : 0;
    if (!ma) sumv = satc = 0;
  } else {
    const bool mb = (__ldg(g.masks + ib) >> sh) & 1u;
    uint32_t boundary = s;
    while (boundary < s + GS && item_index(g, boundary) == ia) ++boundary;
#pragma unroll
    for (int i = 0; i < GS; ++i) {
      const bool m = (s + i) >= boundary ? mb : ma;
      const float vf = static_cast<float>(v[i]);
      out[i] = gate_value(vf, b, m);
      if (dc && m) res += out[i] - vf;
      cnt += m;
      sumv += m ? v[i] : 0;
      satc += m && ((v[i] == lo) | (v[i] == hi));
    }
  }
  if (stats) {
    if (gate) {
      st.n1 += cnt;
      st.s1 += sumv;
      st.sat1 += satc;
    } else {
      st.n0 += cnt;
      st.s0 += sumv;
      st.sat0 += satc;
    }
    if (dc && cnt) {
      dc->s += sumv;
      dc->n += cnt;
      dc->r += res;
    }
  }
}

// One gate of one group of both pols: re[] = pol 0, im[] = pol 1.  The pols
// share the sample index, hence the (merged dual-pol) item and its masks, and
// the heap pair: pol 1's bytes lie one heap after pol 0's.  Statistics of
// pol 0 go to st0 and of pol 1 to st1 when `stats` is set.
template <int NBITS, int GS = Group<NBITS>::samples>
__device__ __forceinline__ void gate_group_dual(const GateParams& g, uint32_t s, float b0, float b1, int gate,
                                                float (&re)[GS], float (&im)[GS], GateStats& st0, GateStats& st1,
                                                bool stats, DcAcc* dc0 = nullptr, DcAcc* dc1 = nullptr) {
  const uint32_t byte0 = static_cast<uint32_t>(static_cast<uint64_t>(s) * NBITS / 8);
  const uint32_t h = heap_of(g, byte0);
  const uint8_t* p0 = g.block + 2ull * h * g.heap_size + (byte0 - h * g.heap_size);
  int v0[GS], v1[GS];
  unpack_span<NBITS, GS>(p0, v0, g.win16 != 0);
  unpack_span<NBITS, GS>(p0 + g.heap_size, v1, g.win16 != 0);
  const uint32_t ia = item_index(g, s);
  const uint32_t ib = item_index(g, s + GS - 1);
  const uint32_t sh = gate ? 1u : 0u;
  const bool ma = (__ldg(g.masks + ia) >> sh) & 1u;
  constexpr int lo = -(1 << (NBITS - 1)), hi = (1 << (NBITS - 1)) - 1;
  int sum0 = 0, sum1 = 0, sat0 = 0, sat1 = 0, cnt = 0;
  float r0 = 0.f, r1 = 0.f;
  if (ib == ia) {
#pragma unroll
    for (int i = 0; i < GS; ++i) {
      const float f0 = static_cast<float>(v0[i]), f1 = static_cast<float>(v1[i]);
      re[i] = gate_value(f0, b0, ma);
      im[i] = gate_value(f1, b1, ma);
      if (dc0) {
        r0 += re[i] - f0;
        r1 += im[i] - f1;
      }
      sum0 += v0[i];
      sum1 += v1[i];
      sat0 += (v0[i] == lo) | (v0[i] == hi);
      sat1 += (v1[i] == lo) | (v1[i] == hi);
    }
    cnt = ma ? GS : 0;
    if (!ma) sum0 = sum1 = sat0 = sat1 = 0;
  } else {
    const bool mb = (__ldg(g.masks + ib) >> sh) & 1u;
    uint32_t boundary = s;
    while (boundary < s + GS && item_index(g, boundary) == ia) ++boundary;
#pragma unroll
    for (int i = 0; i < GS; ++i) {
      const bool m = (s + i) >= boundary ? mb : ma;
      const float f0 = static_cast<float>(v0[i]), f1 = static_cast<float>(v1[i]);
      re[i] = gate_value(f0, b0, m);
      im[i] = gate_value(f1, b1, m);
      if (dc0 && m) {
        r0 += re[i] - f0;
        r1 += im[i] - f1;
      }
      cnt += m;
      sum0 += m ? v0[i] : 0;
      sum1 += m ? v1[i] : 0;
      sat0 += m && ((v0[i] == lo) | (v0[i] == hi));
      sat1 += m && ((v1[i] == lo) | (v1[i] == hi));
    }
  }
  if (dc0 && stats && cnt) {
    dc0->s += sum0;
    dc0->n += cnt;
    dc0->r += r0;
    dc1->s += sum1;
    dc1->n += cnt;
    dc1->r += r1;
  }
  if (stats) {
    if (gate) {
      st0.n1 += cnt;
      st0.s1 += sum0;
      st0.sat1 += sat0;
      st1.n1 += cnt;
      st1.s1 += sum1;
      st1.sat1 += sat1;
    } else {
      st0.n0 += cnt;
      st0.s0 += sum0;
      st0.sat0 += sat0;
      st1.n0 += cnt;
      st1.s0 += sum1;
      st1.sat0 += sat1;
    }
  }
}

// ------------------------------------------------------------------ jobs
// A job is one complex FFT of two real sequences packed as z = a + i b.
//   single pol: a = gate gA of frame fA, b = gate gB of frame fB (or zero);
//               a frame with data in both gates is one job (f,0)+(f,1),
//               frames with data in one gate are paired two per job;
//   dual pol:   a = pol 0, b = pol 1 of gate gA of frame fA.
// Gates without any sample in a frame are constant (their baseline) and
// contribute only to bin 0, counted in dc[gate].
// Encoding: fA | gA << 14 | fB << 16 | gB << 30, fB == kNoFrame: no b.
constexpr uint32_t kNoFrame = 0x3FFFu;
constexpr uint32_t kMaxJobFrames = 0x3FFFu;

__host__ __device__ __forceinline__ uint32_t job_pack(uint32_t fa, uint32_t ga, uint32_t fb, uint32_t gb) {
  return fa | (ga << 14) | (fb << 16) | (gb << 30);
}
__device__ __forceinline__ uint32_t job_fa(uint32_t j) { return j & 0x3FFFu; }
__device__ __forceinline__ uint32_t job_ga(uint32_t j) { return (j >> 14) & 1u; }
__device__ __forceinline__ uint32_t job_fb(uint32_t j) { return (j >> 16) & 0x3FFFu; }
__device__ __forceinline__ uint32_t job_gb(uint32_t j) { return (j >> 30) & 1u; }

// Builds the job list of nf frames whose gate flags (bit0 gate 0 has data,
// bit1 gate 1 has data) are flags[0..nf); frame numbers in the jobs are
// relative to flags.  Returns the number of jobs; dc[g] receives the number
// of frames whose gate g holds no data.  Run by one thread.
__device__ __forceinline__ uint32_t build_jobs(const uint8_t* flags, uint32_t nf, bool dual, uint32_t* jobs,
                                               uint32_t (&dc)[2]) {
  uint32_t n = 0;
  dc[0] = dc[1] = 0;
  uint32_t pend = kNoFrame, pend_g = 0;
  for (uint32_t f = 0; f < nf; ++f) {
    const uint32_t fl = flags[f];
    const bool a0 = fl & 1u, a1 = fl & 2u;
    dc[0] += !a0;
    dc[1] += !a1;
    if (dual) {
      if (a0) jobs[n++] = job_pack(f, 0, kNoFrame, 0);
      if (a1) jobs[n++] = job_pack(f, 1, kNoFrame, 0);
    } else if (a0 && a1) {
      jobs[n++] = job_pack(f, 0, f, 1);
    } else if (a0 || a1) {
      const uint32_t gsel = a1 ? 1u : 0u;
      if (pend == kNoFrame) {
        pend = f;
        pend_g = gsel;
      } else {
        jobs[n++] = job_pack(pend, pend_g, f, gsel);
        pend = kNoFrame;
      }
    }
  }
  if (pend != kNoFrame) jobs[n++] = job_pack(pend, pend_g, kNoFrame, 0);
  return n;
}

}  // namespace gspec
