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
// split into kMaxParts parts (BF16 or FP16 bit patterns; part q is the
// rounding of what parts 0..q-1 left of the FP64 value), stored as
// parts[q * 4096 + 64 n + k]; and the 1024 twiddles W1024^j =
// exp(-2 pi i j / 1024) in FP32 from FP64.
__global__ void tables_kernel(uint16_t* parts, float2* w1024, int bf16) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 64 * 64; i += gridDim.x * blockDim.x) {
    const int n = i >> 6, k = i & 63;
    const int c = n >> 1, s = n & 1, a = k >> 1, r = k & 1;
    double sn, cs;
    sincospi(2.0 * ((a * c) & 31) / 32.0, &sn, &cs);
    double v = (s == 0) ? (r == 0 ? cs : sn) : (r == 0 ? -sn : cs);
    for (int q = 0; q < kMaxParts; ++q) {
      if (bf16) {
        const __nv_bfloat16 h = __double2bfloat16(v);
        parts[q * 4096 + i] = *reinterpret_cast<const uint16_t*>(&h);
        v -= static_cast<double>(__bfloat162float(h));
      } else {
        const __half h = __double2half(v);
        parts[q * 4096 + i] = *reinterpret_cast<const uint16_t*>(&h);
        v -= static_cast<double>(__half2float(h));
      }
    }
  }
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < 1024; j += gridDim.x * blockDim.x) {
    double sn, cs;
    sincospi(2.0 * j / 1024.0, &sn, &cs);
    w1024[j] = make_float2(static_cast<float>(cs), static_cast<float>(-sn));
  }
}

cudaError_t launch_tables(uint16_t* parts, float2* w1024, bool bf16, cudaStream_t s) {
  tables_kernel<<<16, 256, 0, s>>>(parts, w1024, bf16 ? 1 : 0);
  return cudaGetLastError();
}

// The shared-memory image of [B1 | B2 | B3 | W1024] (canonical layout, pad
// bytes zero; the twiddles as the [c][lane] table of stage_tw) that every
// tensor-core CTA copies with 16-byte loads.
__global__ void image_kernel(const uint16_t* parts, const float2* w, uint8_t* img) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < static_cast<int>(kImageBytes); i += gridDim.x * blockDim.x)
    img[i] = 0;
  __syncthreads();
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < 64 * 64; i += gridDim.x * blockDim.x) {
    const int n = i >> 6, k = i & 63;
    for (int q = 0; q < kMaxParts; ++q)
      *reinterpret_cast<uint16_t*>(img + q * kBBytes + kmaj_off(n, k)) = parts[q * 4096 + i];
  }
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < 1024; j += gridDim.x * blockDim.x)
    reinterpret_cast<float2*>(img + kMaxParts * kBBytes)[stage_tw(j & 31, j >> 5)] = w[(j & 31) * (j >> 5)];
}

cudaError_t launch_image(const uint16_t* parts, const float2* w, uint8_t* img, cudaStream_t s) {
  image_kernel<<<1, 256, 0, s>>>(parts, w, img);
  return cudaGetLastError();
}

// Test kernel: ntiles x 4 transforms of 1024 points, global in/out.
template <bool BF16>
__global__ void __launch_bounds__(128) dft1024_test_kernel(const float2* __restrict__ in, float2* __restrict__ out,
                                                           const uint16_t* __restrict__ g_parts,
                                                           const float2* __restrict__ g_w, uint32_t* err) {
  extern __shared__ __align__(1024) char smem[];
  TileSmem s;
  for (int q = 0; q < kMaxParts; ++q) {
    s.a[q] = smem + q * kABytes;
    s.b[q] = smem + kMaxParts * kABytes + q * kBBytes;
  }
  float2* w = reinterpret_cast<float2*>(smem + kMaxParts * (kABytes + kBBytes));
  float2* xs = w + 1024;                                         // 4 x 1024 inputs, then outputs
  uint64_t* bar = reinterpret_cast<uint64_t*>(xs + 4 * 1024);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 1);
  s.w = w;
  s.bar = bar;
  const int tid = threadIdx.x;
  load_dft32_operand(s.b, g_parts, tid, 128);
  for (int i = tid; i < 1024; i += 128) w[stage_tw(i & 31, i >> 5)] = g_w[(i & 31) * (i >> 5)];
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
  const bool ok = dft1024_tile<Split<BF16>>(
      s, phase, tid, [&](int t, int n) { return xs[t * 1024 + n]; },
      [&](int t, int k, float2 v) { out[(static_cast<size_t>(blockIdx.x) * 4 + t) * 1024 + k] = v; }, [] {});
  if (!ok && err) atomicExch(err, 3u);
  __syncthreads();
  fence_after();
  if (tid < 32) tmem_dealloc(s.tmem, kCols);
}

size_t test_smem_bytes() { return kMaxParts * (kABytes + kBBytes) + 1024 * 8 + 4 * 1024 * 8 + 16; }

}  // namespace tc
}  // namespace gspec

using namespace gspec;

extern "C" int gspec_tc_dft1024_device(const void* d_in, void* d_out, uint32_t ntransforms, int form,
                                       void* cuda_stream) {
  if (!d_in || !d_out || ntransforms == 0 || ntransforms % 4) return GSPEC_ERR_ARG;
  if (form != GSPEC_FORM_BF16 && form != GSPEC_FORM_FP16) return GSPEC_ERR_ARG;
  const bool bf16 = form == GSPEC_FORM_BF16;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  uint16_t* parts = nullptr;
  float2* w = nullptr;
  uint32_t* err = nullptr;
  int rc = GSPEC_OK;
  if (cudaMalloc(&parts, tc::kMaxParts * 4096 * 2) != cudaSuccess ||
      cudaMalloc(&w, 1024 * sizeof(float2)) != cudaSuccess || cudaMalloc(&err, 4) != cudaSuccess) {
    rc = GSPEC_ERR_CUDA;
  } else {
    cudaMemsetAsync(err, 0, 4, s);
    tc::launch_tables(parts, w, bf16, s);
    const size_t smem = tc::test_smem_bytes();
    auto kern = bf16 ? tc::dft1024_test_kernel<true> : tc::dft1024_test_kernel<false>;
    cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    kern<<<ntransforms / 4, 128, smem, s>>>(static_cast<const float2*>(d_in), static_cast<float2*>(d_out), parts, w,
                                             err);
    uint32_t h_err = 0;
    if (cudaGetLastError() != cudaSuccess || cudaMemcpyAsync(&h_err, err, 4, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
      rc = GSPEC_ERR_CUDA;
    else if (h_err)
      rc = GSPEC_ERR_CUDA;
  }
  cudaFree(parts);
  cudaFree(w);
  cudaFree(err);
  return rc;
}

// ====================================================================
// Four-step passes of the tensor-core form (N1 = 1024 for pass A, N2 = 1024
// for pass B).  They follow the FP32 passes of gspec_fourstep.cu step by
// step; only the 1024-point FFT of each column / row is replaced by
// dft1024_tile on the tensor cores.
// ====================================================================
#include "gspec_fourstep_common.cuh"

namespace gspec {
namespace tc {

constexpr int kPassThreads = 128;
// Transformed columns of a pass-A tile (written over its operands): column t
// at t * kColStride float2, tile 1's columns kTileSkew float2 further on.  The
// store phase reads (8 columns) x (4 consecutive k1) per warp: with the stride
// = 4 (mod 16) float2 and the skew the 16 lanes of each 8-byte wavefront hit
// distinct banks.
constexpr int kColStride = 1092;
constexpr int kTileSkew = 2;
static_assert(kColStride >= spad_size(1024) && kColStride % 16 == 4, "column stride");
constexpr int kRowStride = spad_size(1024);

// FP16 operand scales (powers of two): pass A inputs are at most 2^11 in
// magnitude, its stage-1 outputs at most 2^11 * 32 * sqrt(2); pass B inputs
// (pass A outputs) at most 2^11 * 1024 * sqrt(2).
// split of each pass: the column pass's first stage transforms integer
// samples, which two parts hold exactly (5 products in BF16); the row pass
// transforms general values (bf16x6 in BF16)
template <bool BF16>
using SplitA = Split<BF16, 2>;
template <bool BF16>
using SplitB = Split<BF16, BF16 ? 3 : 2>;

template <bool BF16> struct Scales {
  static constexpr float a1 = 1.f, a2 = BF16 ? 1.f : 0.25f;
  static constexpr float b1 = BF16 ? 1.f : 1.f / 64, b2 = BF16 ? 1.f : 1.f / 32;
};

__device__ __forceinline__ void load_image(char* dst, const uint4* __restrict__ img, int tid, int nthreads) {
  uint4* d = reinterpret_cast<uint4*>(dst);
  for (int i = tid; i < static_cast<int>(kImageBytes / 16); i += nthreads) d[i] = __ldg(img + i);
}

template <bool BF16>
struct PassALayout {
  static constexpr int BC = 8;                          // columns per CTA: two tiles of 4
  static constexpr int THREADS = 2 * kPassThreads;      // one 128-thread group per tile
  static constexpr size_t A = 0;                        // per tile: operand parts, then its transformed columns
  static constexpr size_t TILE = SplitA<BF16>::n * kABytes;
  static constexpr size_t B = 2 * TILE;                 // [B1 | B2 | B3 | W1024]: the image
  static constexpr size_t RED = B + kImageBytes;
  static constexpr size_t BAR = RED + (THREADS / 32) * 12 * 8;
  static constexpr size_t BYTES = BAR + 32;
  static_assert(static_cast<size_t>(4 * kColStride + kTileSkew) * sizeof(float2) <= TILE, "columns fit the operands");
};

// grid.x = nk * maxjobs * (N2 / 8): (output spectrum, job, 8 columns).  The
// gather unpacks and gates each row's group of samples once and stores the
// 8 kept columns straight into the stage-1 operands of the two tiles; each
// 128-thread group then runs its tile's two tensor-core stages, and the
// transformed columns (written over the operands) leave with the
// W_N^(n2*k1) twiddle.
template <int NBITS, bool DUAL, bool BF16>
__global__ void __launch_bounds__(PassALayout<BF16>::THREADS, SplitA<BF16>::n == 3 ? 1 : 2) tc_a_kernel(FourStepParams p) {
  constexpr int N1 = 1024;
  using L = PassALayout<BF16>;
  constexpr int BC = L::BC, THREADS = L::THREADS;
  constexpr int G = Group<NBITS>::samples;
  constexpr int NPOL = DUAL ? 2 : 1;
  extern __shared__ __align__(1024) char smem[];
  const int tid = threadIdx.x;
  const int grp = tid >> 7, gtid = tid & 127;
  uint64_t* bar = reinterpret_cast<uint64_t*>(smem + L::BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(bar + 2);
  unsigned long long* red = reinterpret_cast<unsigned long long*>(smem + L::RED);
  auto tile_smem = [&](int g) {
    TileSmem t;
    for (int q = 0; q < kMaxParts; ++q) {
      t.a[q] = smem + L::A + g * L::TILE + (q < SplitA<BF16>::n ? q : 0) * kABytes;
      t.b[q] = smem + L::B + q * kBBytes;
    }
    t.w = reinterpret_cast<const float2*>(smem + L::B + kMaxParts * kBBytes);
    t.bar = bar + g;
    return t;
  };
  TileSmem s = tile_smem(grp);
  const TileSmem s0 = tile_smem(0), s1 = tile_smem(1);

  const uint32_t N2 = p.N2;
  const uint32_t N = N1 * N2;
  const uint32_t tiles = N2 / BC;
  const uint32_t tile = blockIdx.x % tiles;
  const uint32_t j = (blockIdx.x / tiles) % p.maxjobs;
  const uint32_t kk = blockIdx.x / (tiles * p.maxjobs);
  const uint32_t k = p.k0 + kk;
  if (j >= p.njobs[k]) return;
  const uint32_t job = p.jobs[k * p.maxjobs + j];
  const uint32_t fa = job_fa(job), ga = job_ga(job), fb = job_fb(job), gb = job_gb(job);
  const uint32_t frA = k * p.c.nacc + fa;
  const uint32_t frB = k * p.c.nacc + fb;
  const uint32_t c0 = tile * BC;

  float bl[2 * NPOL];
#pragma unroll
  for (int i = 0; i < 2 * NPOL; ++i) bl[i] = p.c.baselines[i];
  load_image(smem + L::B, p.tc_img, tid, THREADS);
  if (tid == 0) {
    mbar_init(bar, 1);
    mbar_init(bar + 1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < 32) tmem_alloc(tmem_slot, 2 * kTmemCols);

  // unpack + gate the 8 columns of every row (one group per row) into the
  // stage-1 operands of both tiles
  constexpr float sc1 = Scales<BF16>::a1, sc2 = Scales<BF16>::a2;
  // one span per row: the whole group, or the tile's part of it when that
  // part is whole 32-bit words (12-bit samples)
  constexpr int SP = (G > BC && (BC * NBITS) % 32 == 0) ? BC : G;
  static_assert(SP >= BC, "one span covers the tile's columns");
  const uint32_t gbase = SP <= BC ? c0 : (c0 / SP) * SP;
  const int keep0 = static_cast<int>(c0 - gbase);
  const bool count_stats = SP <= BC || c0 == gbase;
  const uint32_t sg_a = count_stats ? (DUAL ? (1u << ga) : 3u) : 0u;
  static_assert((N1 + THREADS - 1) / THREADS * SP <= 128 && THREADS <= 512,
                "per-thread gate statistics fit the 32-bit commit");
  GateStats st[NPOL];
  DcAcc dc[2];
  // row n1 = 32 a + b goes to operand row b, K pair a (put_stage1): lanes
  // take consecutive a, so that their operand stores hit distinct banks
  static_assert(THREADS == 256 && N1 == 1024, "lanes a = 0..31, b = warp + 8 i");
  for (int i = 0; i < 4; ++i) {
    const int n1 = 32 * (tid & 31) + (tid >> 5) + 8 * i;
    const uint32_t off = N2 * n1 + gbase;
    float re[SP], im[SP];
    if constexpr (DUAL) {
      gate_group_dual<NBITS, SP>(p.c.g, frA * N + off, bl[ga], bl[2 + ga], ga, re, im, st[0], st[NPOL - 1],
                                 count_stats, &dc[0], &dc[1]);
    } else if (fb == fa) {
      gate_group<NBITS, SP>(p.c.g, 0, frA * N + off, bl[0], bl[1], re, im, st[0], sg_a, &dc[0], &dc[1]);
    } else {
      gate_group1<NBITS, SP>(p.c.g, 0, frA * N + off, bl[ga], ga, re, st[0], count_stats, &dc[0]);
      if (fb != kNoFrame) {
        gate_group1<NBITS, SP>(p.c.g, 0, frB * N + off, bl[gb], gb, im, st[0], count_stats, &dc[1]);
      } else {
#pragma unroll
        for (int e = 0; e < SP; ++e) im[e] = 0.f;
      }
    }
#pragma unroll
    for (int e = 0; e < SP; ++e) {
      const int col = e - keep0;
      if (col >= 0 && col < BC) put_stage1<SplitA<BF16>>(col < 4 ? s0 : s1, col & 3, n1, make_float2(re[e], im[e]), sc1);
    }
  }
  fence_before();
  __syncthreads();
  fence_after();
  s.tmem = *tmem_slot + grp * kTmemCols;
  uint32_t phase = 0;
  float2* S = reinterpret_cast<float2*>(s.a[0]) + grp * kTileSkew;   // this tile's columns after the transform
  const bool ok = dft1024_stages<SplitA<BF16>>(
      s, phase, gtid, [&](int t, int k1, float2 v) { S[t * kColStride + spad(k1)] = v; }, [] {}, sc1, sc2);
  if (!ok && gtid == 0 && p.c.dev_err) atomicExch(p.c.dev_err, 3u);
  __syncthreads();
  // twiddle W_N^(n2*k1) and store Y[k1][n2] (as the FP32 pass)
  float2* dst = p.scratch + (static_cast<size_t>(kk) * p.maxjobs + j) * N;
  {
    constexpr int KS = THREADS / BC;
    constexpr int PPT = N1 / KS;
    const int col = tid % BC;
    const uint32_t n2 = c0 + col;
    const float2* Sc = reinterpret_cast<const float2*>(smem + L::A + (col >> 2) * L::TILE) + (col >> 2) * kTileSkew +
                       (col & 3) * kColStride;
    auto exact = [&](uint32_t m) { return cmul(__ldg(&p.twA[m >> 10]), __ldg(&p.twB[m & 1023])); };
    const float2 D = exact(n2 * KS);
    float2 W = make_float2(1.f, 0.f);
#pragma unroll 4
    for (int i = 0; i < PPT; ++i) {
      const int k1 = tid / BC + KS * i;
      W = (i & 3) == 0 ? exact(n2 * static_cast<uint32_t>(k1)) : cmul(W, D);
      dst[static_cast<size_t>(k1) * N2 + n2] = cmul(Sc[spad(k1)], W);
    }
  }
  commit_stats<NPOL>(p.c, st, k, (DUAL ? 8 : 2) * static_cast<int>(N / 2 + 1), red, dc,
                     p.dcsum + (static_cast<size_t>(k) * p.maxjobs + j) * 6);
  fence_after();
  if (tid < 32) tmem_dealloc(*tmem_slot, 2 * kTmemCols);
}

template <bool DUAL, bool BF16>
struct PassBLayout {
  static constexpr int J = 2;                        // jobs per group: 2 jobs x 2 rows = one tile
  static constexpr int VALS = DUAL ? 8 : 2;
  static constexpr int BPT = (1024 + 1 + kPassThreads - 1) / kPassThreads;
  static constexpr size_t A = 0;                     // operand parts; the transformed rows ("work") alias them
  static constexpr size_t B = SplitB<BF16>::n * kABytes;   // [B1 | B2 | B3 | W1024]: the image
  static constexpr size_t W = B + kMaxParts * kBBytes;
  static constexpr size_t JW = W + 1024 * sizeof(float2);
  static constexpr size_t BAR = JW + 16;
  static constexpr size_t BYTES = BAR + 32;
  static_assert(static_cast<size_t>(4) * kRowStride * sizeof(float2) <= SplitB<BF16>::n * kABytes,
                "work fits the operands");
};

// grid.x = nk * N1/2: unit (output spectrum k, row pair rp); jobs two at a
// time.  The first DFT stage reads its operand rows straight from the
// scratch (a warp's loads cover 32 consecutive points of a row), and the next
// group's rows are prefetched into L2 as soon as the first stage has read
// the current ones; without a staging buffer in shared memory two CTAs fit
// an SM in both forms.
template <bool DUAL, bool BF16>
__global__ void __launch_bounds__(kPassThreads, 2) tc_b_kernel(FourStepParams p) {
  constexpr int N2 = 1024;
  using L = PassBLayout<DUAL, BF16>;
  constexpr int J = L::J, BPT = L::BPT, VALS = L::VALS;
  constexpr uint32_t kRowBytes = N2 * sizeof(float2);
  extern __shared__ __align__(1024) char smem[];
  TileSmem s;
  for (int q = 0; q < kMaxParts; ++q) {
    s.a[q] = smem + L::A + (q < SplitB<BF16>::n ? q : 0) * kABytes;
    s.b[q] = smem + L::B + q * kBBytes;
  }
  float2* work = reinterpret_cast<float2*>(smem + L::A);
  float2* w = reinterpret_cast<float2*>(smem + L::W);
  uint32_t* jw = reinterpret_cast<uint32_t*>(smem + L::JW);
  uint64_t* mma_bar = reinterpret_cast<uint64_t*>(smem + L::BAR);
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(mma_bar + 2);
  s.w = w;
  s.bar = mma_bar;

  const uint32_t N1 = p.N1;
  const uint32_t N = N1 * N2;
  const uint32_t C = N / 2 + 1;
  const uint32_t half = N1 / 2;
  const uint32_t kk = blockIdx.x / half;
  const uint32_t k = p.k0 + kk;
  const uint32_t rp = blockIdx.x % half;
  const uint32_t rowA = rp, rowB = rp == 0 ? half : N1 - rp;
  const int nbins = rp == 0 ? N2 + 1 : N2;
  const int tid = threadIdx.x;
  const uint32_t njobs = p.njobs[k];
  const uint32_t* jobs = p.jobs + k * p.maxjobs;
  const uint32_t ngroups = (njobs + J - 1) / J;

  if (tid == 0) {
    mbar_init(mma_bar, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (tid < 32) tmem_alloc(tmem_slot, kTmemCols);
  load_image(smem + L::B, p.tc_img, tid, kPassThreads);
  fence_before();
  __syncthreads();
  fence_after();
  s.tmem = *tmem_slot;

  // the rows of job group g: transform t = 2 qq + r is row rowA (r = 0) or
  // rowB (r = 1) of job g J + qq (the group's last job stands in for a missing one)
  auto row_of = [&](uint32_t g, int t) {
    const uint32_t nq = min(static_cast<uint32_t>(J), njobs - g * J);
    const uint32_t qq = min(static_cast<uint32_t>(t >> 1), nq - 1);
    const float2* seq = p.scratch + (static_cast<size_t>(kk) * p.maxjobs + g * J + qq) * N;
    return seq + static_cast<size_t>((t & 1) ? rowB : rowA) * N2;
  };
  // thread 0: group g's rows into L2
  auto prefetch = [&](uint32_t g) {
    for (int t = 0; t < 2 * J; ++t)
      asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(row_of(g, t)), "r"(kRowBytes) : "memory");
  };
  if (tid == 0 && ngroups > 0) prefetch(0);

  // job words one group ahead: the global load of group g + 1 is in flight
  // while group g is transformed
  uint32_t next_job = (tid < J && static_cast<uint32_t>(tid) < njobs) ? jobs[tid] : 0u;
  float acc[BPT][VALS];
#pragma unroll
  for (int i = 0; i < BPT; ++i)
#pragma unroll
    for (int v = 0; v < VALS; ++v) acc[i][v] = 0.f;

  uint32_t phase = 0;
  bool mma_ok = true;
  for (uint32_t g = 0; g < ngroups; ++g) {
    const uint32_t j0 = g * J;
    const int nq = static_cast<int>(min(static_cast<uint32_t>(J), njobs - j0));
    if (tid < nq) jw[tid] = next_job;
    if (tid < J && j0 + J + tid < njobs) next_job = jobs[j0 + J + tid];
    const float2* my_row = row_of(g, tid >> 5);
    mma_ok = dft1024_tile<SplitB<BF16>>(
                 s, phase, tid, [&](int, int n) { return __ldg(my_row + n); },
                 [&](int t, int k2, float2 v) { work[t * kRowStride + spad(k2)] = v; },
                 [&] {
                   if (tid == 0 && g + 1 < ngroups) prefetch(g + 1);
                 },
                 Scales<BF16>::b1, Scales<BF16>::b2) &&
             mma_ok;
    __syncthreads();
#pragma unroll
    for (int i = 0; i < BPT; ++i) {
      const int a = tid + i * kPassThreads;
      if (a >= nbins) continue;
      int r, k2, pr, k2p;
      pair_slot<N2>(rp, a, r, k2, pr, k2p);
      for (int qq = 0; qq < nq; ++qq) {
        const uint32_t job = jw[qq];
        const float2 za = work[(2 * qq + r) * kRowStride + spad(k2)];
        const float2 zb = work[(2 * qq + pr) * kRowStride + spad(k2p)];
        accumulate_bin<DUAL>(acc[i], za, zb, job);
      }
    }
    __syncthreads();
  }
  if (!mma_ok && tid == 0 && p.c.dev_err) atomicExch(p.c.dev_err, 3u);
  // bin 0 from the exact per-job sums (exact_dc), over the jobs in order;
  // the operand buffers are free after the loop's last barrier
  if (rp == 0)
    exact_dc_bin<DUAL>(p, k, reinterpret_cast<float*>(smem + L::A),
                       static_cast<uint32_t>(SplitB<BF16>::n * kABytes / (VALS * sizeof(float))), acc[0]);
  // gates without data: constant baseline in bin 0 (row pair 0, slot a = 0)
  if (rp == 0 && tid == 0) {
    const float n = static_cast<float>(N);
    for (int gate = 0; gate < 2; ++gate) {
      const float cnt = static_cast<float>(p.dc[2 * k + gate]);
      if (cnt == 0.f) continue;
      if constexpr (!DUAL) {
        const float d = n * p.c.baselines[gate];
        acc[0][gate] += cnt * d * d;
      } else {
        const float x = n * p.c.baselines[gate], y = n * p.c.baselines[2 + gate];
        acc[0][0 + gate] += cnt * (x * x + y * y);
        acc[0][2 + gate] += cnt * (x * x - y * y);
        acc[0][4 + gate] += cnt * (2.f * x * y);
      }
    }
  }
  // row-pair sums, contiguous in the slot a; the scatter kernel adds them to the output
  float* bs = p.bsum + static_cast<size_t>(blockIdx.x) * VALS * (N2 + 1);
  (void)C;
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    const int a = tid + i * kPassThreads;
    if (a >= nbins) continue;
#pragma unroll
    for (int v = 0; v < VALS; ++v) bs[v * (N2 + 1) + a] = acc[i][v];
  }
  fence_after();
  if (tid < 32) tmem_dealloc(s.tmem, kTmemCols);
}

template <class K>
static cudaError_t run_tc(K kern, unsigned grid, size_t smem, const FourStepParams& p, cudaStream_t s,
                          int threads = kPassThreads) {
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  kern<<<grid, threads, smem, s>>>(p);
  return cudaGetLastError();
}

template <bool BF16>
static cudaError_t launch_pass(int pass, int nbits, bool dual, const FourStepParams& p, cudaStream_t s) {
  if (pass == 0) {
    if (p.N1 != 1024) return cudaErrorInvalidValue;
    using LA = PassALayout<BF16>;
    const unsigned grid = p.nk * p.maxjobs * (p.N2 / LA::BC);
    const size_t sm = LA::BYTES;
    switch (nbits * 2 + (dual ? 1 : 0)) {
      case 16: return run_tc(tc_a_kernel<8, false, BF16>, grid, sm, p, s, LA::THREADS);
      case 17: return run_tc(tc_a_kernel<8, true, BF16>, grid, sm, p, s, LA::THREADS);
      case 20: return run_tc(tc_a_kernel<10, false, BF16>, grid, sm, p, s, LA::THREADS);
      case 21: return run_tc(tc_a_kernel<10, true, BF16>, grid, sm, p, s, LA::THREADS);
      case 24: return run_tc(tc_a_kernel<12, false, BF16>, grid, sm, p, s, LA::THREADS);
      case 25: return run_tc(tc_a_kernel<12, true, BF16>, grid, sm, p, s, LA::THREADS);
    }
    return cudaErrorInvalidValue;
  }
  if (p.N2 != 1024) return cudaErrorInvalidValue;
  const unsigned grid = p.nk * (p.N1 / 2);
  return dual ? run_tc(tc_b_kernel<true, BF16>, grid, PassBLayout<true, BF16>::BYTES, p, s)
              : run_tc(tc_b_kernel<false, BF16>, grid, PassBLayout<false, BF16>::BYTES, p, s);
}

cudaError_t launch_tc_pass(int pass, int nbits, bool dual, const FourStepParams& p, cudaStream_t s) {
  return p.form == GSPEC_FORM_FP16 ? launch_pass<false>(pass, nbits, dual, p, s)
                                   : launch_pass<true>(pass, nbits, dual, p, s);
}

}  // namespace tc
}  // namespace gspec
