// Tensor-core (tcgen05) DFT-1024 of the split-precision four-step form.
//
// A 1024-point DFT is two 32-point DFT stages with a twiddle between them
// (n = 32a + b, k = c + 32d):
//   X[c + 32d] = sum_b W32^(bd) * W1024^(bc) * sum_a x[32a + b] W32^(ac).
// Each stage is one real GEMM on the 5th-generation tensor cores: the rows
// are the length-32 sub-sequences of four transforms (4 x 32 = 128 rows, the
// M of one tcgen05.mma), K = 64 real inputs (re, im interleaved), N = 64 real
// outputs (re, im interleaved), with the constant DFT-32 matrix as B.
// Precision: operands are split into parts of the 16-bit type, each part the
// rounding of what the parts before it left (x = x1 + x2 (+ x3) + r), and the
// product is accumulated in FP32 in tensor memory from the partial products
// whose parts together carry the leading bits:
//   FP16 (11-bit parts, two per operand): A1 B1 + A1 B2 + A2 B1, 12 MMAs of
//     K = 16 per stage; what is left is ~2^-22 of the result;
//   BF16 (8-bit parts), three parts per operand: the bf16x6 scheme of Henry,
//     Tang and Heinecke ("Leveraging the bfloat16 artificial intelligence
//     datatype for higher-precision computations", ARITH 2019):
//     A1 B1 + A1 B2 + A2 B1 + A2 B2 + A1 B3 + A3 B1, 24 MMAs per stage,
//     ~2^-24 left over;
//   BF16 with the data operand A in two parts and the constant DFT-32 matrix
//     B in three: A1 B1 + A1 B2 + A2 B1 + A2 B2 + A1 B3 (20 MMAs): exact for
//     data that two parts hold exactly (integer samples up to 2^16), else
//     A's remainder (~2^-18) is left.  The column pass uses it (its first
//     stage transforms integer samples), the row pass uses bf16x6.
// The small products are issued first so that they are summed before the
// large one joins the accumulator.
//
// Shared-memory operands use the canonical K-major layout without swizzle:
// 8-row x 16-byte core matrices; element (row, k) of a bf16 matrix sits at
//   (row / 8) * SBO + (k / 8) * LBO + (row % 8) * 16 + (k % 8) * 2.
// LBO = 144 bytes (not a multiple of 128) keeps the column-wise operand
// stores of the second stage free of bank conflicts.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cstdint>

#include "gspec_device.cuh"

namespace gspec {
namespace tc {

constexpr uint32_t kLBO = 144;
constexpr uint32_t kSBO = 8 * kLBO;              // 8 K-chunks of 8 elements per row group
constexpr uint32_t kABytes = 16 * kSBO;          // 128 rows x 64 bf16
constexpr uint32_t kBBytes = 8 * kSBO;           // 64 rows x 64 bf16
constexpr uint32_t kTmemCols = 64;               // 128 lanes x 64 fp32 accumulators
constexpr int kMaxParts = 3;
constexpr uint32_t kImageBytes = kMaxParts * kBBytes + 1024 * 8;   // [B1 | B2 | B3 | W1024] in shared-memory layout
static_assert(kImageBytes == 3 * 9216 + 1024 * 8, "image size as declared for the host");

// Split policy of one pass: the 16-bit type, the parts of the data operand
// A (n) and the partial products of a stage.  FP16: two parts, 3 products.
// BF16 with n = 3: bf16x6 (6 products); with n = 2 (data exact in two
// parts, e.g. integer samples): A1 B1 + A1 B2 + A2 B1 + A2 B2 + A1 B3
// (5 products).  The DFT-32 matrix B has three parts in BF16, two in FP16.
template <bool BF16_, int NPA_ = (BF16_ ? 3 : 2)>
struct Split {
  static constexpr bool bf16 = BF16_;
  static constexpr int n = NPA_;
  static constexpr int products = !BF16_ ? 3 : (NPA_ == 3 ? 6 : 5);
  static_assert(BF16_ ? (NPA_ == 2 || NPA_ == 3) : NPA_ == 2, "parts of the form");
};
constexpr uint32_t kWaitLimit = 1u << 22;

__host__ __device__ constexpr uint32_t kmaj_off(uint32_t row, uint32_t k) {
  return (row >> 3) * kSBO + (k >> 3) * kLBO + (row & 7) * 16 + (k & 7) * 2;
}

// Shared-memory matrix descriptor: start address, leading (K) and stride
// (row-group) byte offsets, fixed version bits 46-48 = 0b001, no swizzle.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
  return static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4) | (static_cast<uint64_t>(kLBO >> 4) << 16) |
         (static_cast<uint64_t>(kSBO >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: D = F32 (bits 4-5 = 1), A and B BF16
// (bits 7-9, 10-12 = 1) or FP16 (0), both K-major (bits 15, 16 = 0),
// N >> 3 in bits 17-22, M >> 4 in bits 24-28.
__host__ __device__ constexpr uint32_t idesc(int M, int N, bool bf16) {
  return (1u << 4) | ((bf16 ? 1u : 0u) << 7) | ((bf16 ? 1u : 0u) << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
         (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(dst)), "r"(ncols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t id, uint32_t accumulate) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(id), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void commit(uint64_t* bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
               : "memory");
}

// 32 consecutive fp32 columns of this thread's TMEM lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// Split of a complex value into SP::n packed 16-bit pairs (re in the low
// half): part i is the rounding of what parts 0..i-1 left; every remainder
// is exact in FP32.
template <class SP>
__device__ __forceinline__ void splitn(float2 v, uint32_t (&p)[SP::n]) {
#pragma unroll
  for (int i = 0; i < SP::n; ++i) {
    if constexpr (SP::bf16) {
      const __nv_bfloat162 h = __floats2bfloat162_rn(v.x, v.y);
      const float2 hf = __bfloat1622float2(h);
      p[i] = *reinterpret_cast<const uint32_t*>(&h);
      v = make_float2(v.x - hf.x, v.y - hf.y);
    } else {
      const __half2 h = __floats2half2_rn(v.x, v.y);
      const float2 hf = __half22float2(h);
      p[i] = *reinterpret_cast<const uint32_t*>(&h);
      v = make_float2(v.x - hf.x, v.y - hf.y);
    }
  }
}

// Shared memory of one tile engine (offsets from a 1024-byte aligned base).
struct TileSmem {
  char* a[kMaxParts];   // operand parts, kABytes each (the pass uses SP::n)
  char* b[kMaxParts];   // DFT-32 matrix parts, kBBytes each
  const float2* w;      // stage twiddles: W1024^(lane*c) at stage_tw(lane, c)
  uint64_t* bar;        // MMA completion barrier
  uint32_t tmem;        // TMEM base (kTmemCols columns)
};

// The twiddle between the DFT-32 stages of row (t, lane), output c is
// W1024^(lane*c).  Stored as a [c][lane] table (the 1024 values of W1024 in
// another order, lane * c < 1024), the 32 lanes that read output c take 32
// consecutive entries: no bank conflicts, where the natural order W1024[lane*c]
// made lanes collide in gcd(c, 16) ways.
__host__ __device__ constexpr int stage_tw(int lane, int c) { return c * 32 + lane; }

// (A part, B part) of the partial products of a stage, smallest first:
// 6 products (2,0) (0,2) (1,1) (1,0) (0,1) (0,0); 5 products (1,1) (0,2)
// (1,0) (0,1) (0,0); 3 products (1,0) (0,1) (0,0).
template <class SP>
__host__ __device__ constexpr int prod_a(int q) {
  return SP::products == 6 ? (q == 0 ? 2 : q == 2 ? 1 : q == 3 ? 1 : 0)
         : SP::products == 5 ? (q == 0 ? 1 : q == 2 ? 1 : 0)
                             : (q == 0 ? 1 : 0);
}
template <class SP>
__host__ __device__ constexpr int prod_b(int q) {
  return SP::products == 6 ? (q == 1 ? 2 : q == 2 ? 1 : q == 4 ? 1 : 0)
         : SP::products == 5 ? (q == 0 ? 1 : q == 1 ? 2 : q == 3 ? 1 : 0)
                             : (q == 1 ? 1 : 0);
}

// Issues one stage (the pass's partial products over K = 64, 4 MMAs of
// K = 16 each, the smallest products first) and a commit.
template <class SP>
__device__ __forceinline__ void issue_stage(const TileSmem& s) {
  constexpr uint32_t id = idesc(128, 64, SP::bf16);
  constexpr int NPROD = SP::products;
  fence_after();
#pragma unroll
  for (int q = 0; q < NPROD; ++q) {
    const uint32_t a = smem_addr(s.a[prod_a<SP>(q)]), b = smem_addr(s.b[prod_b<SP>(q)]);
#pragma unroll
    for (uint32_t ks = 0; ks < 4; ++ks) {
      const uint32_t off = ks * 2 * kLBO;
      mma(s.tmem, sdesc(a + off), sdesc(b + off), id, (q > 0 || ks > 0) ? 1u : 0u);
    }
  }
  commit(s.bar);
}

__device__ __forceinline__ float2 scale2(float2 v, float f) { return make_float2(v.x * f, v.y * f); }

// Stage-1 operand of input x[t][n] (n = 32a + b) in row 32t + b, K = 2a + r,
// stored by whoever produces the value (scaled by sc1, split hi/lo).
template <class SP>
__device__ __forceinline__ void put_stage1(const TileSmem& s, int t, int n, float2 v, float sc1) {
  uint32_t p[SP::n];
  splitn<SP>(scale2(v, sc1), p);
  const uint32_t off = kmaj_off(32 * t + (n & 31), 2 * (n >> 5));
#pragma unroll
  for (int i = 0; i < SP::n; ++i) *reinterpret_cast<uint32_t*>(s.a[i] + off) = p[i];
}

// The two tensor-core stages of a tile whose stage-1 operands are in place
// (see dft1024_tile); every thread of the block calls it.
template <class SP, class Y, class M>
__device__ __forceinline__ bool dft1024_stages(const TileSmem& s, uint32_t& phase, int tid, Y y, M mid, float sc1,
                                               float sc2) {
  const int t = tid >> 5, lane = tid & 31;
  fence_async_smem();
  __syncthreads();
  mid();
  if (tid == 0) issue_stage<SP>(s);
  bool ok = mbar_wait(s.bar, phase, kWaitLimit);
  phase ^= 1u;
  fence_after();
  const uint32_t lane_addr = s.tmem + (static_cast<uint32_t>(t * 32) << 16);
  float v[32];
  {
    // outputs c = 0..15 (columns 0..31), twiddled, into the stage-2 rows (t, c)
    tmem_ld32(lane_addr, v);
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const float2 z = scale2(cmul(make_float2(v[2 * c], v[2 * c + 1]), s.w[stage_tw(lane, c)]), sc2);
      uint32_t p[SP::n];
      splitn<SP>(z, p);
#pragma unroll
      for (int i = 0; i < SP::n; ++i)
        *reinterpret_cast<uint32_t*>(s.a[i] + kmaj_off(32 * t + c, 2 * lane)) = p[i];
    }
    tmem_ld32(lane_addr + 32, v);
#pragma unroll
    for (int c = 0; c < 16; ++c) {
      const float2 z = scale2(cmul(make_float2(v[2 * c], v[2 * c + 1]), s.w[stage_tw(lane, c + 16)]), sc2);
      uint32_t p[SP::n];
      splitn<SP>(z, p);
#pragma unroll
      for (int i = 0; i < SP::n; ++i)
        *reinterpret_cast<uint32_t*>(s.a[i] + kmaj_off(32 * t + c + 16, 2 * lane)) = p[i];
    }
  }
  fence_before();
  fence_async_smem();
  __syncthreads();
  if (tid == 0) issue_stage<SP>(s);
  ok = mbar_wait(s.bar, phase, kWaitLimit) && ok;
  phase ^= 1u;
  fence_after();
  // stage 2: row tid = (t, c = lane) holds X[c + 32d], d = 0..31
  const float inv = 1.f / (sc1 * sc2);
  tmem_ld32(lane_addr, v);
#pragma unroll
  for (int d = 0; d < 16; ++d) y(t, lane + 32 * d, make_float2(v[2 * d] * inv, v[2 * d + 1] * inv));
  tmem_ld32(lane_addr + 32, v);
#pragma unroll
  for (int d = 0; d < 16; ++d) y(t, lane + 32 * (d + 16), make_float2(v[2 * d] * inv, v[2 * d + 1] * inv));
  fence_before();
  return ok;
}

// DFT-1024 of four transforms by the 128 threads of the calling group
// (thread tid of the group; all threads of the block call it together).
// x(t, n) returns input n of transform t; y(t, k, v) takes output k.
// mid() runs on every thread once the inputs have been read (after the
// first barrier), e.g. to start loading the next inputs.  sc1 and sc2 scale
// the operands of the two stages by powers of two (the FP16 form keeps them
// in range); the outputs are scaled back exactly.  Returns false if a
// bounded wait on the tensor cores gave up.
template <class SP, class X, class Y, class M>
__device__ __forceinline__ bool dft1024_tile(const TileSmem& s, uint32_t& phase, int tid, X x, Y y, M mid,
                                             float sc1 = 1.f, float sc2 = 1.f) {
  const int t = tid >> 5, lane = tid & 31;
  // stage 1: row tid = (t, b = lane) holds x[32a + b], a = 0..31
  constexpr int NP = SP::n;
#pragma unroll
  for (int kc = 0; kc < 8; ++kc) {
    uint32_t p[4][NP];
#pragma unroll
    for (int j = 0; j < 4; ++j) splitn<SP>(scale2(x(t, 32 * (4 * kc + j) + lane), sc1), p[j]);
#pragma unroll
    for (int i = 0; i < NP; ++i)
      *reinterpret_cast<uint4*>(s.a[i] + kmaj_off(tid, 8 * kc)) = make_uint4(p[0][i], p[1][i], p[2][i], p[3][i]);
  }
  return dft1024_stages<SP>(s, phase, tid, y, mid, sc1, sc2);
}

// Copies the DFT-32 operand parts (kMaxParts logical [n][k] 64 x 64 16-bit
// arrays, one after the other in global memory) into the canonical layout.
__device__ __forceinline__ void load_dft32_operand(char* const (&b)[kMaxParts], const uint16_t* g_parts, int tid,
                                                   int nthreads) {
  for (int i = tid; i < 64 * 64; i += nthreads) {
    const int n = i >> 6, k = i & 63;
#pragma unroll
    for (int q = 0; q < kMaxParts; ++q) *reinterpret_cast<uint16_t*>(b[q] + kmaj_off(n, k)) = g_parts[q * 4096 + i];
  }
}

}  // namespace tc
}  // namespace gspec
