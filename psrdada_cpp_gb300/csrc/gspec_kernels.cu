// Gated-spectrometer kernels for sm_103a.
//
// Small FFT lengths (N <= 4096) run the whole chain of one frame inside one
// CTA: unpack + gate (edd/src/Unpacker.cu:24-108, edd/src/GatedSpectrometer.cu:22-59)
// into shared memory, one complex Stockham FFT per pair of real sequences
// (replacing the two cuFFT R2C calls, edd/detail/GatedSpectrometer.cu:281-288),
// and the detect (edd/DetectorAccumulator.cuh:40-61) or Stokes
// (edd/src/GatedSpectrometer.cu:140-169) accumulation fused into the epilogue.
//
// Two real sequences a, b share one complex FFT of z = a + i b:
//   A(k) = (Z(k) + conj Z(N-k)) / 2 ,  B(k) = (Z(k) - conj Z(N-k)) / (2i).
// Which sequences are paired is decided per frame from the side-channel
// gates (build_jobs): only gates holding data are transformed; a gate
// without data is the constant baseline and adds to bin 0 only.
#include <algorithm>

#include "gspec_kernels.cuh"

// Twiddle tables of the shared-memory path: 1 copies them to shared memory,
// 0 reads them through the read-only cache.
#ifndef GSPEC_SMALL_TW_SMEM
#define GSPEC_SMALL_TW_SMEM 0
#endif

// Programmatic dependent launch of the warp chain after the gate pre-pass.
#ifndef GSPEC_PDL
#define GSPEC_PDL 1
#endif

namespace gspec {

// ------------------------------------------------------------------ helpers
__device__ __forceinline__ unsigned long long warp_sum_u64(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Reduce NV per-thread values over the block; thread v < NV of the block
// receives total v in `out` (returns true for those threads).
template <int NV>
__device__ __forceinline__ bool block_sum_u64(unsigned long long (&vals)[NV], unsigned long long* red,
                                             unsigned long long& out) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int v = 0; v < NV; ++v) {
    unsigned long long s = warp_sum_u64(vals[v]);
    if (lane == 0) red[warp * NV + v] = s;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    unsigned long long s = 0;
    for (int w = 0; w < nwarps; ++w) s += red[w * NV + threadIdx.x];
    out = s;
  }
  return threadIdx.x < NV;
}

// Add the block's gate statistics to the counters.
//   per pol: n0, n1, s0, s1 -> pol_stats;  sum over pols: n0, n1 -> output
//   record counters of spectrum k; sat0, sat1 -> sat[k].
template <int NPOL>
__device__ __forceinline__ void commit_stats(const ChainParams& p, const GateStats (&st)[NPOL], uint32_t k,
                                             int vals_c, unsigned long long* red, bool store_counts = false) {
  constexpr int NV = 4 * NPOL + 4;
  unsigned long long v[NV];
#pragma unroll
  for (int q = 0; q < NPOL; ++q) {
    v[4 * q + 0] = st[q].n0;
    v[4 * q + 1] = st[q].n1;
    v[4 * q + 2] = static_cast<unsigned long long>(st[q].s0);
    v[4 * q + 3] = static_cast<unsigned long long>(st[q].s1);
  }
  unsigned long long n0 = 0, n1 = 0, s0 = 0, s1 = 0;
#pragma unroll
  for (int q = 0; q < NPOL; ++q) {
    n0 += st[q].n0;
    n1 += st[q].n1;
    s0 += st[q].sat0;
    s1 += st[q].sat1;
  }
  v[4 * NPOL + 0] = n0;
  v[4 * NPOL + 1] = n1;
  v[4 * NPOL + 2] = s0;
  v[4 * NPOL + 3] = s1;
  unsigned long long tot;
  if (block_sum_u64<NV>(v, red, tot)) {
    const int i = threadIdx.x;
    if (i < 4 * NPOL) {
      if (tot) atomicAdd(p.pol_stats + i, tot);
    } else {
      const int j = i - 4 * NPOL;
      if (j < 2) {
        unsigned long long* cnt =
            reinterpret_cast<unsigned long long*>(p.out + k * p.out_rec + static_cast<uint64_t>(vals_c) * 4);
        // store_counts: this CTA holds all of spectrum k's frames of an output
        // that one block fills, so its counts are the record's counters
        if (store_counts) {
          cnt[j] = tot;
        } else if (tot) {
          atomicAdd(cnt + j, tot);
        }
      } else {
        if (tot) atomicAdd(p.sat + 2 * k + (j - 2), tot);
      }
    }
  }
  __syncthreads();
}

// ------------------------------------------------------------ small chain
template <int N, bool DUAL>
struct SmallCfg {
  static constexpr int P = 16;
  static constexpr int T = N / P;                 // threads per FFT
  static constexpr int NSLOT = T >= 256 ? 1 : 256 / T;
  static constexpr int THREADS = NSLOT * T;
  // a slot's sequence and accumulator are touched by its own threads only,
  // so a round needs the slot's barrier only: its warp (T <= 32) or a named
  // barrier of its T threads (id 1 + slot), the CTA when one slot fills it
  static constexpr int SYNC = T <= 32 ? kSyncWarp : (NSLOT > 1 ? kSyncNamed : kSyncCta);
  static_assert(SYNC != kSyncNamed || NSLOT <= 15, "named barrier ids 1..15");
  static constexpr int C = N / 2 + 1;
  static constexpr int VALS = DUAL ? 8 : 2;
  static constexpr int SEQ_F2 = spad_size(N);
  static constexpr int MAX_JOBS = 2 * kMaxUnitFrames;
  static constexpr size_t SEQ_BYTES = static_cast<size_t>(NSLOT) * SEQ_F2 * sizeof(float2);
  static constexpr size_t ACC_BYTES = static_cast<size_t>(NSLOT) * VALS * C * sizeof(float);
  static constexpr size_t RED_BYTES = static_cast<size_t>(THREADS / 32) * 12 * sizeof(unsigned long long);
  static constexpr size_t JOB_BYTES = (MAX_JOBS + 4) * sizeof(uint32_t);
  static constexpr size_t TW_BYTES = static_cast<size_t>(tw_size(N)) * sizeof(float2);
  static constexpr size_t SMEM = SEQ_BYTES + ACC_BYTES + RED_BYTES + JOB_BYTES + TW_BYTES;
};

// One CTA per work unit (output spectrum k, slice of its frames).  The
// unit's job list (build_jobs) is worked through NSLOT jobs at a time; each
// slot accumulates its jobs' spectra in shared memory; slots are summed in
// a fixed order at the end, so results do not depend on scheduling.
#ifndef GSPEC_SMALL_MINB
#define GSPEC_SMALL_MINB 2   // resident CTAs per SM the register allocation is sized for
#endif
template <int N, int NBITS, bool DUAL>
__global__ void __launch_bounds__(SmallCfg<N, DUAL>::THREADS, GSPEC_SMALL_MINB)
    small_chain_kernel(ChainParams p) {
  using Cfg = SmallCfg<N, DUAL>;
  constexpr int G = Group<NBITS>::samples;
  constexpr int NG = N / G;
  constexpr int C = Cfg::C;
  constexpr int NPOL = DUAL ? 2 : 1;
  static_assert(N % G == 0, "frame must hold whole unpack groups");

  extern __shared__ float4 smem_f4[];
  char* base = reinterpret_cast<char*>(smem_f4);
  float2* S = reinterpret_cast<float2*>(base);
  float* acc = reinterpret_cast<float*>(base + Cfg::SEQ_BYTES);
  unsigned long long* red = reinterpret_cast<unsigned long long*>(base + Cfg::SEQ_BYTES + Cfg::ACC_BYTES);
  uint32_t* jobs = reinterpret_cast<uint32_t*>(base + Cfg::SEQ_BYTES + Cfg::ACC_BYTES + Cfg::RED_BYTES);
  uint32_t* jinfo = jobs + Cfg::MAX_JOBS;   // [0] njobs, [1] dc gate 0, [2] dc gate 1
  float2* tws = reinterpret_cast<float2*>(base + Cfg::SEQ_BYTES + Cfg::ACC_BYTES + Cfg::RED_BYTES + Cfg::JOB_BYTES);

  const int tid = threadIdx.x;
  const int slot = tid / Cfg::T;
  const int t = tid - slot * Cfg::T;

  const uint32_t unit = blockIdx.x;
  const uint32_t k = unit / p.slices;
  const uint32_t sl = unit - k * p.slices;
  const uint32_t f0 = k * p.nacc + sl * p.frames_per_unit;

  if (tid == 0) {
    uint32_t dc[2];
    jinfo[0] = build_jobs(p.flags + f0, p.frames_per_unit, DUAL, jobs, dc);
    jinfo[1] = dc[0];
    jinfo[2] = dc[1];
  }
  float bl[2 * NPOL];
#pragma unroll
  for (int i = 0; i < 2 * NPOL; ++i) bl[i] = p.baselines[i];
  for (int i = tid; i < Cfg::NSLOT * Cfg::VALS * C; i += Cfg::THREADS) acc[i] = 0.f;
#if GSPEC_SMALL_TW_SMEM
  load_twiddles<N>(tws, p.tw);
  const float2* twp = tws;
#else
  const float2* twp = p.tw;
#endif
  __syncthreads();
  const uint32_t njobs = jinfo[0];

  GateStats st[NPOL];
  float2* Z = S + slot * Cfg::SEQ_F2;
  float* A = acc + slot * Cfg::VALS * C;
  auto round_sync = [&] { group_sync<Cfg::SYNC>(1 + slot, Cfg::T); };

  for (uint32_t it = 0; it < njobs; it += Cfg::NSLOT) {
    const uint32_t jx = it + slot;
    const bool active = jx < njobs;
    const uint32_t job = active ? jobs[jx] : 0u;
    const uint32_t fa = job_fa(job), ga = job_ga(job), fb = job_fb(job), gb = job_gb(job);
    if (active) {
      // spans of SP samples: whole 32-bit words from a group start (8 samples
      // at 8 and 12 bits, 16 at 10 bits), so a thread holds fewer values than
      // a whole 16- or 32-sample group would take
      constexpr int SP = NBITS == 10 ? 16 : 8;
      static_assert(G % SP == 0 && (SP * NBITS) % 32 == 0, "spans are whole words within a group");
#pragma unroll 1
      for (int gi = t; gi < N / SP; gi += Cfg::T) {
        const uint32_t sa = (f0 + fa) * N + gi * SP;
        float re[SP], im[SP];
        if constexpr (DUAL) {
          gate_group_dual<NBITS, SP>(p.g, sa, bl[ga], bl[2 + ga], ga, re, im, st[0], st[NPOL - 1], true);
        } else if (fb == fa) {
          gate_group<NBITS, SP>(p.g, 0, sa, bl[0], bl[1], re, im, st[0], 3u);
        } else {
          gate_group1<NBITS, SP>(p.g, 0, sa, bl[ga], ga, re, st[0], true);
          if (fb != kNoFrame) {
            gate_group1<NBITS, SP>(p.g, 0, (f0 + fb) * N + gi * SP, bl[gb], gb, im, st[0], true);
          } else {
#pragma unroll
            for (int e = 0; e < SP; ++e) im[e] = 0.f;
          }
        }
#pragma unroll
        for (int e = 0; e < SP; ++e) Z[spad(gi * SP + e)] = make_float2(re[e], im[e]);
      }
    }
    {
      // the next round's samples of this slot into L2 while this round is transformed
      const uint32_t jn = it + Cfg::NSLOT + slot;
      if (jn < njobs) {
        const uint32_t job_n = jobs[jn];
        const uint32_t fan = job_fa(job_n), fbn = job_fb(job_n);
#pragma unroll 1
        for (int gi = t; gi < NG; gi += Cfg::T) {
          const uint64_t byte0 = static_cast<uint64_t>((f0 + fan) * N + gi * G) * NBITS / 8;
          prefetch_l2(pol_byte(p.g, 0, byte0));
          if constexpr (DUAL) {
            prefetch_l2(pol_byte(p.g, 1, byte0));
          } else if (fbn != fan && fbn != kNoFrame) {
            prefetch_l2(pol_byte(p.g, 0, static_cast<uint64_t>((f0 + fbn) * N + gi * G) * NBITS / 8));
          }
        }
      }
    }
    round_sync();
    fft_smem<N, Cfg::P, 1, Cfg::SYNC>(Z, twp, t, active, 1 + slot);
    if (active) {
#pragma unroll 1
      for (int c = t; c < C; c += Cfg::T) {
        const float2 a = Z[spad(c)], b = Z[spad((N - c) & (N - 1))];
        if constexpr (!DUAL) {
          // A = Z(c), B = conj Z(N-c): |A+B|^2/4 and |A-B|^2/4
          const float sx = a.x + b.x, sy = a.y - b.y;
          const float dx = a.x - b.x, dy = a.y + b.y;
          A[ga * C + c] += 0.25f * fmaf(sx, sx, sy * sy);
          if (fb != kNoFrame) A[gb * C + c] += 0.25f * fmaf(dx, dx, dy * dy);
        } else {
          const float p1x = 0.5f * (a.x + b.x), p1y = 0.5f * (a.y - b.y);
          const float p2x = 0.5f * (a.y + b.y), p2y = -0.5f * (a.x - b.x);
          const float a1 = fmaf(p1x, p1x, p1y * p1y);
          const float a2 = fmaf(p2x, p2x, p2y * p2y);
          A[(0 + ga) * C + c] += a1 + a2;
          A[(2 + ga) * C + c] += a1 - a2;
          A[(4 + ga) * C + c] += 2.f * fmaf(p1x, p2x, p1y * p2y);
          A[(6 + ga) * C + c] += -2.f * fmaf(p1y, p2x, -p1x * p2y);
        }
      }
    }
    round_sync();
  }
  __syncthreads();
  // gates without data in a frame: constant baseline, bin 0 only
  if (tid == 0) {
    const float n = static_cast<float>(N);
    for (int gate = 0; gate < 2; ++gate) {
      const float cnt = static_cast<float>(jinfo[1 + gate]);
      if (cnt == 0.f) continue;
      if constexpr (!DUAL) {
        const float d = n * bl[gate];
        acc[gate * C] += cnt * d * d;
      } else {
        const float x = n * bl[gate], y = n * bl[2 + gate];
        acc[(0 + gate) * C] += cnt * (x * x + y * y);
        acc[(2 + gate) * C] += cnt * (x * x - y * y);
        acc[(4 + gate) * C] += cnt * (2.f * x * y);
      }
    }
  }
  __syncthreads();

  // slots -> output (fixed order)
  float* outf = reinterpret_cast<float*>(p.out + k * p.out_rec);
  for (int i = tid; i < Cfg::VALS * C; i += Cfg::THREADS) {
    float v = 0.f;
#pragma unroll 4
    for (int s = 0; s < Cfg::NSLOT; ++s) v += acc[s * Cfg::VALS * C + i];
    if (p.slices == 1) {
      outf[i] = p.store ? v : outf[i] + v;
    } else {
      p.partial[(static_cast<size_t>(k) * p.slices + sl) * Cfg::VALS * C + i] = v;
    }
  }
  commit_stats<NPOL>(p, st, k, Cfg::VALS * C, red);
}

// Block finalisation (counters, baselines of the next block, error-word
// mirror); `red` holds 2 x (warps of the CTA) 64-bit words of shared memory.
__device__ void finalize_block(const ChainParams& p, int npol, int C, int dual, int convention, int ungated,
                               float* baselines_out, unsigned long long* red);

// ------------------------------------------------------------ warp chain
// Single-pol 1024-point chain with one FFT per warp (N = 32 x 32).  Lane l
// unpacks and gates the 32 consecutive samples 32 l .. 32 l + 31 of each of
// the job's two frames (one item lookup per span, as in the shared-memory
// chain) into two padded 32 x 33 float planes of the warp's tile; reading
// them back by column leaves z[32 j + l] (j = 0..31) in lane l.  A DFT-32
// over j in registers, a multiply by W1024^(l k1), and a transpose through
// the same tile give lane k1 row k1 for the second DFT-32: lane k1 ends with
// Z(k1 + 32 k2), k2 = 0..31, and the mirror Z(N - c) of its bin c comes
// from lane (32 - k1) mod 32 by one shuffle.  A warp works through its
// jobs on its own (no block barrier in the job loop), holding its bins'
// power sums in registers; the warps' sums are added in a fixed order at the
// end, so results do not depend on scheduling.

// W32^c = exp(-2 pi i c / 32), c = 0..15, from cos/sin of pi/16, pi/8, 3 pi/16, pi/4
constexpr float kC16 = 0.98078528040323044913f, kS16 = 0.19509032201612826785f;   // cos, sin pi/16
constexpr float kC316 = 0.83146961230254523708f, kS316 = 0.55557023301960222474f; // cos, sin 3pi/16
__device__ __forceinline__ float2 w32(int c) {
  switch (c) {
    case 1: return make_float2(kC16, -kS16);
    case 2: return make_float2(kC8, -kS8);
    case 3: return make_float2(kC316, -kS316);
    case 4: return make_float2(kS2, -kS2);
    case 5: return make_float2(kS316, -kC316);
    case 6: return make_float2(kS8, -kC8);
    case 7: return make_float2(kS16, -kC16);
    case 9: return make_float2(-kS16, -kC16);
    case 10: return make_float2(-kS8, -kC8);
    case 11: return make_float2(-kS316, -kC316);
    case 12: return make_float2(-kS2, -kS2);
    case 13: return make_float2(-kC316, -kS316);
    case 14: return make_float2(-kC8, -kS8);
    default: return make_float2(-kC16, -kS16);   // 15
  }
}

// Forward DFT-32 in registers, natural order in and out: DFT-16 of the even
// and the odd samples, then X[c] = E[c] + W32^c O[c], X[c + 16] = E[c] - W32^c O[c].
__device__ __forceinline__ void dft32(float2 (&v)[32]) {
  float2 e[16], o[16];
#pragma unroll
  for (int b = 0; b < 16; ++b) {
    e[b] = v[2 * b];
    o[b] = v[2 * b + 1];
  }
  dft16(e);
  dft16(o);
#pragma unroll
  for (int c = 0; c < 16; ++c) {
    const float2 t = c == 0 ? o[0] : (c == 8 ? cmul_mi(o[8]) : cmul(o[c], w32(c)));
    v[c] = cadd(e[c], t);
    v[c + 16] = csub(e[c], t);
  }
}

struct WarpChainCfg {
  static constexpr int N = 1024, C = N / 2 + 1;
  static constexpr int WARPS = 8, THREADS = 32 * WARPS;
  static constexpr int TILE = 32 * 33;                                  // float2 per warp tile
  static constexpr size_t TILE_BYTES = static_cast<size_t>(WARPS) * TILE * sizeof(float2);
  static constexpr size_t TW_BYTES = 1024 * sizeof(float2);
  static constexpr int MAX_JOBS = 2 * kMaxUnitFrames;
  static constexpr size_t JOB_BYTES = (MAX_JOBS + 4) * sizeof(uint32_t);
  static constexpr size_t RED_BYTES = WARPS * 12 * sizeof(unsigned long long);
  static constexpr size_t SMEM = TILE_BYTES + TW_BYTES + JOB_BYTES + RED_BYTES;
  static_assert(static_cast<size_t>(WARPS) * 2 * C * sizeof(float) <= TILE_BYTES, "warp sums fit the tiles");
};

template <int NBITS>
__global__ void __launch_bounds__(WarpChainCfg::THREADS, 2) warp_chain_kernel(ChainParams p) {
  using Cfg = WarpChainCfg;
  constexpr int N = Cfg::N, C = Cfg::C;
  extern __shared__ float4 smem_f4[];
  char* base = reinterpret_cast<char*>(smem_f4);
  float2* tiles = reinterpret_cast<float2*>(base);
  float2* tw = reinterpret_cast<float2*>(base + Cfg::TILE_BYTES);                 // [k1][lane]
  uint32_t* jobs = reinterpret_cast<uint32_t*>(base + Cfg::TILE_BYTES + Cfg::TW_BYTES);
  uint32_t* jinfo = jobs + Cfg::MAX_JOBS;   // [0] njobs, [1] dc gate 0, [2] dc gate 1
  unsigned long long* red =
      reinterpret_cast<unsigned long long*>(base + Cfg::TILE_BYTES + Cfg::TW_BYTES + Cfg::JOB_BYTES);

  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const uint32_t unit = blockIdx.x;
  const uint32_t k = unit / p.slices;
  const uint32_t sl = unit - k * p.slices;
  const uint32_t f0 = k * p.nacc + sl * p.frames_per_unit;
  // the stage twiddles W1024^(lane k1) follow the Stockham tables of N
  for (int i = tid; i < 1024; i += Cfg::THREADS) tw[i] = __ldg(p.tw + tw_size(N) + i);
#if GSPEC_PDL
  // launched as a programmatic dependent of the gate pre-pass: its masks and
  // frame flags are complete once this returns
  asm volatile("griddepcontrol.wait;" ::: "memory");
#endif
  if (tid == 0) {
    uint32_t dc[2];
    jinfo[0] = build_jobs(p.flags + f0, p.frames_per_unit, false, jobs, dc);
    jinfo[1] = dc[0];
    jinfo[2] = dc[1];
  }
  const float b0 = p.baselines[0], b1 = p.baselines[1];
  __syncthreads();
  const uint32_t njobs = jinfo[0];
  GateStats st;
  float acc0[17], acc1[17];
#pragma unroll
  for (int i = 0; i < 17; ++i) acc0[i] = acc1[i] = 0.f;
  float2* T = tiles + warp * Cfg::TILE;

  for (uint32_t jx = warp; jx < njobs; jx += Cfg::WARPS) {
    const uint32_t job = jobs[jx];
    const uint32_t fa = job_fa(job), ga = job_ga(job), fb = job_fb(job), gb = job_gb(job);
    const bool has_b = fb != kNoFrame;
    const float ba = ga ? b1 : b0, bb = gb ? b1 : b0;
    // frame a (gate ga) into the re plane, frame b (gate gb; a job of one
    // frame with data in both gates has fb == fa) into the im plane
    float* Tre = reinterpret_cast<float*>(T);
    float* Tim = Tre + 32 * 33;
#pragma unroll 1
    for (int h = 0; h < 2; ++h) {
      float v[32];
      if (h == 0 || has_b) {
        const uint32_t s0 = (f0 + (h ? fb : fa)) * N + 32 * lane;
        gate_group1<NBITS, 32>(p.g, 0, s0, h ? bb : ba, h ? gb : ga, v, st, true);
      } else {
#pragma unroll
        for (int j = 0; j < 32; ++j) v[j] = 0.f;
      }
      float* P = h ? Tim : Tre;
#pragma unroll
      for (int j = 0; j < 32; ++j) P[lane * 33 + j] = v[j];
    }
    __syncwarp();
    float2 x[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) x[j] = make_float2(Tre[j * 33 + lane], Tim[j * 33 + lane]);
    __syncwarp();
    // DFT-32 over j; twiddle W1024^(lane k1); transpose through the warp's tile
    dft32(x);
#pragma unroll
    for (int k1 = 1; k1 < 32; ++k1) x[k1] = cmul(x[k1], tw[k1 * 32 + lane]);
#pragma unroll
    for (int k1 = 0; k1 < 32; ++k1) T[k1 * 33 + lane] = x[k1];
    __syncwarp();
#pragma unroll
    for (int n2 = 0; n2 < 32; ++n2) x[n2] = T[lane * 33 + n2];
    __syncwarp();
    // DFT-32 over n2: lane k1 holds Z(k1 + 32 k2) in x[k2]
    dft32(x);
    // bins c = lane + 32 k2 <= N/2, the mirror Z(N - c) from lane (32 - lane) mod 32
    // (lane 0: its own x[(32 - k2) mod 32]); A = (Z(c) + conj Z(N-c))/2, B = (Z(c) - conj Z(N-c))/(2i)
    const int partner = (32 - lane) & 31;
#pragma unroll
    for (int k2 = 0; k2 < 17; ++k2) {
      const float2 src = x[31 - (k2 & 15) - (k2 >> 4) * 16];
      float2 b = make_float2(__shfl_sync(0xffffffffu, src.x, partner), __shfl_sync(0xffffffffu, src.y, partner));
      if (lane == 0) b = x[(32 - k2) & 31];
      if (k2 == 16 && lane != 0) continue;
      const float2 a = x[k2];
      const float sx = a.x + b.x, sy = a.y - b.y;
      const float dx = a.x - b.x, dy = a.y + b.y;
      const float pa = 0.25f * fmaf(sx, sx, sy * sy);
      const float pb = has_b ? 0.25f * fmaf(dx, dx, dy * dy) : 0.f;
      acc0[k2] += (ga == 0 ? pa : 0.f) + (gb == 0 ? pb : 0.f);
      acc1[k2] += (ga != 0 ? pa : 0.f) + (gb != 0 ? pb : 0.f);
    }
  }
  __syncthreads();
  // the warps' sums, then their fixed-order total; the tiles are free now
  float* wsum = reinterpret_cast<float*>(tiles);   // [warp][2][C]
#pragma unroll
  for (int k2 = 0; k2 < 17; ++k2) {
    const int c = lane + 32 * k2;
    if (c > N / 2) continue;
    wsum[(warp * 2 + 0) * C + c] = acc0[k2];
    wsum[(warp * 2 + 1) * C + c] = acc1[k2];
  }
  __syncthreads();
  float* outf = reinterpret_cast<float*>(p.out + k * p.out_rec);
  const float n = static_cast<float>(N);
  for (int i = tid; i < 2 * C; i += Cfg::THREADS) {
    float v = 0.f;
#pragma unroll
    for (int w = 0; w < Cfg::WARPS; ++w) v += wsum[w * 2 * C + i];
    // gates without data in a frame: constant baseline, bin 0 only
    if (i == 0 || i == C) {
      const int gate = i == 0 ? 0 : 1;
      const float cnt = static_cast<float>(jinfo[1 + gate]);
      if (cnt != 0.f) {
        const float d = n * (gate ? b1 : b0);
        v += cnt * d * d;
      }
    }
    if (p.slices == 1) {
      outf[i] = p.store ? v : outf[i] + v;
    } else {
      p.partial[(static_cast<size_t>(k) * p.slices + sl) * 2 * C + i] = v;
    }
  }
  GateStats sts[1] = {st};
  commit_stats<1>(p, sts, k, 2 * C, red, p.store && p.slices == 1);
  if (p.ticket) {
    // the last CTA to finish runs the block finalisation: every CTA makes its
    // outputs and counters visible device-wide before it takes its ticket
    __threadfence();
    __syncthreads();
    if (tid == 0) jinfo[3] = atomicInc(p.ticket, gridDim.x - 1) == gridDim.x - 1 ? 1u : 0u;
    __syncthreads();
    if (jinfo[3]) {
      __threadfence();
      finalize_block(p, 1, C, 0, p.fin_convention, p.fin_ungated, p.fin_baselines, red);
    }
  }
}

// Pre-pass of a block: the gate masks of every side-channel item index of
// one pol (dual: merged items; bit0 gate 0, bit1 gate 1), and per frame the
// gates holding at least one sample.  The items a frame touches are
// item_index(first) .. item_index(last) in steps of nsc (the index is
// monotonic inside a gating chunk and frames never straddle chunks).
__global__ void gate_prepass_kernel(GateParams g, uint32_t nitems, uint8_t* masks, uint32_t N, uint32_t nframes,
                                    uint8_t* flags, uint32_t L) {
#if GSPEC_PDL
  // a programmatic dependent (the warp chain) may start its prologue now; it
  // waits for this grid's completion before it reads masks or flags
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
#endif
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nitems; i += stride) {
    bool m0, m1;
    item_masks(load_item(g, i), g.bitpos, m0, m1);
    masks[i] = static_cast<uint8_t>(m0 | (m1 << 1));
  }
  if (!flags) return;
  // L lanes per frame (a power of two up to 32, about the items a frame
  // spans: 256 at 2^20 samples and 4096-sample heaps, 1 at 1024 samples);
  // the warp loop is uniform so that every lane takes part in the shuffles
  const uint32_t lane = threadIdx.x & 31;
  const uint32_t fpw = 32 / L;
  const uint32_t f_sub = lane / L, sub = lane & (L - 1);
  for (uint32_t w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; w * fpw < nframes; w += stride >> 5) {
    const uint32_t f = w * fpw + f_sub;
    uint32_t fl = 0;
    if (f < nframes) {
      const uint32_t i0 = item_index(g, f * N), i1 = item_index(g, f * N + N - 1);
      for (uint32_t i = i0 + sub * g.nsc; i <= i1; i += L * g.nsc) {
        bool m0, m1;
        item_masks(load_item(g, i), g.bitpos, m0, m1);
        fl |= m0 | (m1 << 1);
      }
    }
    for (uint32_t o = L / 2; o > 0; o >>= 1) fl |= __shfl_xor_sync(0xffffffffu, fl, o);
    if (f < nframes && sub == 0) flags[f] = static_cast<uint8_t>(fl);
  }
}

// Baselines for the next block (edd/src/GatedSpectrometer.cu:98-118), with
// exact integer sums, an FP64 division and a zero-count guard; then the
// Stokes record's counter copies (edd/src/GatedSpectrometer.cu:485-525),
// and the device error word into its page-locked host mirror.  Run by every
// thread of one CTA after every counter of the block is final.
__device__ void finalize_block(const ChainParams& p, int npol, int C, int dual, int convention, int ungated,
                               float* baselines_out, unsigned long long* red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = (blockDim.x + 31) >> 5;
  const int vals = dual ? 8 : 2;
  unsigned long long t0 = 0, t1 = 0;
  for (uint32_t k = threadIdx.x; k < p.n_out; k += blockDim.x) {
    const unsigned long long* cnt =
        reinterpret_cast<const unsigned long long*>(p.out + k * p.out_rec + static_cast<uint64_t>(vals) * C * 4);
    t0 += cnt[0];
    t1 += cnt[1];
  }
  t0 = warp_sum_u64(t0);
  t1 = warp_sum_u64(t1);
  if (lane == 0) {
    red[2 * warp] = t0;
    red[2 * warp + 1] = t1;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    t0 = t1 = 0;
    for (int w = 0; w < nwarps; ++w) {
      t0 += red[2 * w];
      t1 += red[2 * w + 1];
    }
    for (int pol = 0; pol < npol; ++pol) {
      unsigned long long* ps = p.pol_stats + pol * kPolStats;
      unsigned long long den0 = ps[0], den1 = ps[1];
      if (convention == 1) {
        // cumulative output counters at the time this pol's update ran
        den0 = t0;
        den1 = t1;
        if (npol == 2 && pol == 0) {
          den0 -= p.pol_stats[kPolStats + 0];
          den1 -= p.pol_stats[kPolStats + 1];
        }
      }
      const long long s0 = static_cast<long long>(ps[2]);
      const long long s1 = static_cast<long long>(ps[3]);
      // ungated: no gate, no baseline ((v - 0) + 0 = v for the next block)
      baselines_out[2 * pol + 0] =
          (den0 && !ungated) ? static_cast<float>(static_cast<double>(s0) / static_cast<double>(den0)) : 0.f;
      baselines_out[2 * pol + 1] =
          (den1 && !ungated) ? static_cast<float>(static_cast<double>(s1) / static_cast<double>(den1)) : 0.f;
    }
    for (int i = 0; i < npol * kPolStats; ++i) p.pol_stats[i] = 0;
    // the error word of the block's kernels (all of them ran before this one)
    if (p.err_host) *p.err_host = *p.dev_err;
  }
  if (dual) {
    for (uint32_t k = threadIdx.x; k < p.n_out; k += blockDim.x) {
      unsigned long long* cnt =
          reinterpret_cast<unsigned long long*>(p.out + k * p.out_rec + static_cast<uint64_t>(vals) * C * 4);
      const unsigned long long c0 = cnt[0], c1 = cnt[1];
      for (int r = 1; r < 4; ++r) {
        cnt[2 * r] = c0;
        cnt[2 * r + 1] = c1;
      }
    }
  }
}

__global__ void finalize_kernel(ChainParams p, int npol, int C, int dual, int convention, int ungated,
                                float* baselines_out) {
  __shared__ unsigned long long red[2 * 32];
  finalize_block(p, npol, C, dual, convention, ungated, baselines_out, red);
}

// out[k][i] += sum_s partial[k][s][i] (fixed order); the last block of the
// grid also runs the block finalisation (the counters are final already).
__global__ void reduce_finalize_kernel(ChainParams p, int vals_c, int npol, int C, int dual, int convention,
                                       int ungated, float* baselines_out) {
  const uint32_t k = blockIdx.y;
  float* outf = reinterpret_cast<float*>(p.out + k * p.out_rec);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < vals_c; i += gridDim.x * blockDim.x) {
    float v = 0.f;
    const float* src = p.partial + static_cast<size_t>(k) * p.slices * vals_c + i;
    for (uint32_t s = 0; s < p.slices; ++s) v += src[static_cast<size_t>(s) * vals_c];
    outf[i] = p.store ? v : outf[i] + v;
  }
  __shared__ unsigned long long red[2 * 32];
  if (blockIdx.x == gridDim.x - 1 && blockIdx.y == gridDim.y - 1)
    finalize_block(p, npol, C, dual, convention, ungated, baselines_out, red);
}

// --------------------------------------------------------------- twiddles
// FP64 twiddles (sincospi) rounded once to FP32.
__global__ void twiddle_pass_kernel(float2* tw, int ns, int r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= ns * r) return;
  const int kk = i / ns, q = i - kk * ns;
  double s, c;
  sincospi(-2.0 * static_cast<double>(q) * kk / (static_cast<double>(ns) * r), &s, &c);
  tw[i] = make_float2(static_cast<float>(c), static_cast<float>(s));
}

__global__ void twiddle_split_kernel(float2* twA, float2* twB, int N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int nhi = (N + 1023) / 1024;
  double s, c;
  if (i < 1024) {
    sincospi(-2.0 * static_cast<double>(i) / N, &s, &c);
    twB[i] = make_float2(static_cast<float>(c), static_cast<float>(s));
  }
  if (i < nhi) {
    sincospi(-2.0 * static_cast<double>(i) * 1024.0 / N, &s, &c);
    twA[i] = make_float2(static_cast<float>(c), static_cast<float>(s));
  }
}

// ------------------------------------------------------------ debug / unpack
template <int NBITS>
__global__ void gate_debug_kernel(GateParams g, const float* baselines, int npol, uint32_t nsamps, float* out) {
  constexpr int G = Group<NBITS>::samples;
  const uint32_t ngroups = nsamps / G;
  for (uint32_t gi = blockIdx.x * blockDim.x + threadIdx.x; gi < ngroups; gi += gridDim.x * blockDim.x) {
    const uint32_t s = gi * G;
    for (int pol = 0; pol < npol; ++pol) {
      float a0[G], a1[G];
      GateStats st;
      gate_group<NBITS>(g, pol, s, baselines[2 * pol], baselines[2 * pol + 1], a0, a1, st);
      float* o0 = out + static_cast<size_t>(2 * pol) * nsamps + s;
      float* o1 = out + static_cast<size_t>(2 * pol + 1) * nsamps + s;
#pragma unroll
      for (int e = 0; e < G; ++e) {
        o0[e] = a0[e];
        o1[e] = a1[e];
      }
    }
  }
}

template <int NBITS>
__global__ void unpack_kernel(const uint8_t* raw, uint64_t ngroups, float* out) {
  constexpr int G = Group<NBITS>::samples;
  constexpr int GB = Group<NBITS>::words * 8;
  for (uint64_t gi = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; gi < ngroups;
       gi += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    int v[G];
    unpack_group<NBITS>(raw + gi * GB, v);
#pragma unroll
    for (int e = 0; e < G; ++e) out[gi * G + e] = static_cast<float>(v[e]);
  }
}

// ------------------------------------------------------------ dispatch
template <int N, bool DUAL>
static cudaError_t launch_small_t(int nbits, const ChainParams& p, cudaStream_t s) {
  using Cfg = SmallCfg<N, DUAL>;
  const unsigned grid = p.n_out * p.slices;
  auto run = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(Cfg::SMEM));
    if (e != cudaSuccess) return e;
    kern<<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(p);
    return cudaGetLastError();
  };
  switch (nbits) {
    case 8: return run(small_chain_kernel<N, 8, DUAL>);
    case 10: return run(small_chain_kernel<N, 10, DUAL>);
    case 12: return run(small_chain_kernel<N, 12, DUAL>);
  }
  return cudaErrorInvalidValue;
}

template <bool DUAL>
static cudaError_t launch_small_d(int N, int nbits, const ChainParams& p, cudaStream_t s) {
  switch (N) {
    case 32: return launch_small_t<32, DUAL>(nbits, p, s);
    case 64: return launch_small_t<64, DUAL>(nbits, p, s);
    case 128: return launch_small_t<128, DUAL>(nbits, p, s);
    case 256: return launch_small_t<256, DUAL>(nbits, p, s);
    case 512: return launch_small_t<512, DUAL>(nbits, p, s);
    case 1024: return launch_small_t<1024, DUAL>(nbits, p, s);
    case 2048: return launch_small_t<2048, DUAL>(nbits, p, s);
    case 4096: return launch_small_t<4096, DUAL>(nbits, p, s);
  }
  return cudaErrorInvalidValue;
}

bool small_fft_supported(int N) { return N >= 32 && N <= 4096 && (N & (N - 1)) == 0; }

template <bool DUAL>
static void small_cfg_query(int N, int& threads, size_t& smem) {
#define GSPEC_Q(NN)                          \
  case NN:                                   \
    threads = SmallCfg<NN, DUAL>::THREADS;   \
    smem = SmallCfg<NN, DUAL>::SMEM;         \
    return;
  switch (N) {
    GSPEC_Q(32) GSPEC_Q(64) GSPEC_Q(128) GSPEC_Q(256) GSPEC_Q(512) GSPEC_Q(1024) GSPEC_Q(2048) GSPEC_Q(4096)
  }
#undef GSPEC_Q
  threads = 0;
  smem = 0;
}

int small_fft_threads(int N, bool dual) {
  int t;
  size_t s;
  if (dual) small_cfg_query<true>(N, t, s); else small_cfg_query<false>(N, t, s);
  return t;
}

size_t small_fft_smem(int N, bool dual) {
  int t;
  size_t s;
  if (dual) small_cfg_query<true>(N, t, s); else small_cfg_query<false>(N, t, s);
  return s;
}

template <int NBITS>
static cudaError_t launch_warp_chain_t(const ChainParams& p, cudaStream_t s) {
  using Cfg = WarpChainCfg;
  auto kern = warp_chain_kernel<NBITS>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(Cfg::SMEM));
  if (e != cudaSuccess) return e;
#if GSPEC_PDL
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(p.n_out * p.slices);
  cfg.blockDim = dim3(Cfg::THREADS);
  cfg.dynamicSmemBytes = Cfg::SMEM;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, kern, p);
#else
  kern<<<p.n_out * p.slices, Cfg::THREADS, Cfg::SMEM, s>>>(p);
  return cudaGetLastError();
#endif
}

cudaError_t launch_small_chain(int N, int nbits, bool dual, const ChainParams& p, cudaStream_t s) {
  // single-pol 1024-point frames: one FFT per warp (warp_chain_kernel)
  if (uses_warp_chain(N, dual)) {
    switch (nbits) {
      case 8: return launch_warp_chain_t<8>(p, s);
      case 10: return launch_warp_chain_t<10>(p, s);
      case 12: return launch_warp_chain_t<12>(p, s);
    }
    return cudaErrorInvalidValue;
  }
  return dual ? launch_small_d<true>(N, nbits, p, s) : launch_small_d<false>(N, nbits, p, s);
}

cudaError_t launch_reduce_finalize(int N, bool dual, const ChainParams& p, int npol, int convention, int ungated,
                                   float* baselines_out, cudaStream_t s) {
  const int C = N / 2 + 1;
  const int vals_c = (dual ? 8 : 2) * C;
  dim3 grid((vals_c + 255) / 256, p.n_out);
  reduce_finalize_kernel<<<grid, 256, 0, s>>>(p, vals_c, npol, C, dual ? 1 : 0, convention, ungated, baselines_out);
  return cudaGetLastError();
}

cudaError_t launch_prepass(const GateParams& g, uint32_t nitems, uint8_t* masks, uint32_t N, uint32_t nframes,
                           uint8_t* flags, cudaStream_t s) {
  // lanes per frame: the items a frame spans, as a power of two up to 32
  const uint64_t span = (static_cast<uint64_t>(N) * g.nbits / 8 + g.heap_size - 1) / std::max<uint64_t>(g.heap_size, 1);
  uint32_t L = 1;
  while (L < 32 && L < span) L <<= 1;
  const uint64_t work = std::max<uint64_t>(nitems, static_cast<uint64_t>(nframes) * L);
  const unsigned grid = static_cast<unsigned>(std::min<uint64_t>(4 * 152, (work + 255) / 256));
  gate_prepass_kernel<<<grid ? grid : 1, 256, 0, s>>>(g, nitems, masks, N, nframes, flags, L);
  return cudaGetLastError();
}

cudaError_t launch_finalize(const ChainParams& p, int npol, int C, int dual, int convention, int ungated,
                            float* baselines_out, cudaStream_t s) {
  finalize_kernel<<<1, 256, 0, s>>>(p, npol, C, dual, convention, ungated, baselines_out);
  return cudaGetLastError();
}

// W1024^(lane k1) at [k1 * 32 + lane] (lane, k1 < 32), in FP64 and rounded once.
__global__ void warp_stage_twiddle_kernel(float2* tw) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 1024) return;
  const int k1 = i >> 5, lane = i & 31;
  double sn, cs;
  sincospi(-2.0 * static_cast<double>(lane * k1) / 1024.0, &sn, &cs);
  tw[i] = make_float2(static_cast<float>(cs), static_cast<float>(sn));
}

cudaError_t launch_twiddles(int N, float2* tw, cudaStream_t s) {
  if (N == 1024) {
    warp_stage_twiddle_kernel<<<4, 256, 0, s>>>(tw + tw_size(N));
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  for (int ns = 1; ns < N; ns *= pass_radix(N, ns)) {
    const int r = pass_radix(N, ns);
    if (ns == 1) continue;
    const int off = tw_offset(N, ns);
    const int n = ns * r;
    twiddle_pass_kernel<<<(n + 255) / 256, 256, 0, s>>>(tw + off, ns, r);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_fourstep_twiddles(int N, float2* twA, float2* twB, cudaStream_t s) {
  twiddle_split_kernel<<<4, 256, 0, s>>>(twA, twB, N);
  return cudaGetLastError();
}

cudaError_t launch_gate_debug(int nbits, const GateParams& g, const float* baselines, int npol, uint32_t nsamps,
                              float* out, cudaStream_t s) {
  const int grid = 4 * 152, block = 256;
  switch (nbits) {
    case 8: gate_debug_kernel<8><<<grid, block, 0, s>>>(g, baselines, npol, nsamps, out); break;
    case 10: gate_debug_kernel<10><<<grid, block, 0, s>>>(g, baselines, npol, nsamps, out); break;
    case 12: gate_debug_kernel<12><<<grid, block, 0, s>>>(g, baselines, npol, nsamps, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_unpack(int nbits, const uint8_t* raw, uint64_t nsamples, float* out, cudaStream_t s) {
  const int grid = 4 * 152, block = 256;
  switch (nbits) {
    case 8: unpack_kernel<8><<<grid, block, 0, s>>>(raw, nsamples / Group<8>::samples, out); break;
    case 10: unpack_kernel<10><<<grid, block, 0, s>>>(raw, nsamples / Group<10>::samples, out); break;
    case 12: unpack_kernel<12><<<grid, block, 0, s>>>(raw, nsamples / Group<12>::samples, out); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Mirrors the device error word into host memory (page-locked, device
// accessible) with one store from an SM: no copy engine is involved, so the
// status of a block never waits behind other streams' bulk copies.

// Copies between device memory and page-locked host memory with SM loads and
// stores (small blocks of the serving loop, which then never queue behind
// other streams' bulk copies on the copy engines).  8-byte words for any
// 8-byte multiple; 16-byte words with four loads in flight per thread before
// the stores when both ends are 16-byte aligned, because loads from host
// memory over the chip-to-chip link take microseconds.
__global__ void copy_words_kernel(const uint2* __restrict__ src, uint2* dst, uint64_t n) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n; i += stride) dst[i] = src[i];
}

__global__ void copy_quads_kernel(const uint4* src, uint4* dst, uint64_t n) {
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x;
  for (; i + 3 * stride < n; i += 4 * stride) {
    const uint4 a = src[i], b = src[i + stride], c = src[i + 2 * stride], d = src[i + 3 * stride];
    dst[i] = a;
    dst[i + stride] = b;
    dst[i + 2 * stride] = c;
    dst[i + 3 * stride] = d;
  }
  for (; i < n; i += stride) dst[i] = src[i];
}

cudaError_t launch_copy_words(void* dst, const void* src, uint64_t bytes, int sm_count, cudaStream_t s) {
  if (bytes % 8 || (reinterpret_cast<uintptr_t>(dst) | reinterpret_cast<uintptr_t>(src)) % 8)
    return cudaErrorInvalidValue;   // 8-byte words only
  const bool quads = bytes % 16 == 0 && reinterpret_cast<uintptr_t>(dst) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(src) % 16 == 0;
  const uint64_t n = bytes / (quads ? 16 : 8);
  // 32 CTAs of 256 threads with four 16-byte loads in flight per thread
  // already fill the host link both ways (208 GB/s in, 191 GB/s out on
  // GB300): the copy holds few CTA slots and the chains of other streams
  // keep the rest
  uint64_t blocks = (n + 255) / 256;
  const uint64_t cap = sm_count < 32 ? static_cast<uint64_t>(sm_count) : 32ull;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  if (quads)
    copy_quads_kernel<<<static_cast<unsigned>(blocks), 256, 0, s>>>(static_cast<const uint4*>(src),
                                                                   static_cast<uint4*>(dst), n);
  else
    copy_words_kernel<<<static_cast<unsigned>(blocks), 256, 0, s>>>(static_cast<const uint2*>(src),
                                                                   static_cast<uint2*>(dst), n);
  return cudaGetLastError();
}

}  // namespace gspec
