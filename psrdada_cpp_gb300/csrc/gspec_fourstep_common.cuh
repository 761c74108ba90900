// Pieces shared by the FP32 four-step passes (gspec_fourstep.cu) and the
// tensor-core passes (gspec_tc.cu).
#pragma once

#include "gspec_kernels.cuh"

namespace gspec {

// Same commit rule as the shared-memory path: per-pol n0, n1, s0, s1 to
// pol_stats; n0, n1 summed over pols to the output record; saturation to sat[k].
// A pass-A thread gathers at most four groups of at most 32 samples per pol
// (|sample| <= 2048, so |sum| <= 2^18), and a CTA has at most 512 threads:
// its counts and sums fit in 32 bits and each warp reduces them with one
// redux.sync per value.
//
// With dc_out (the job's 6 DC slots), the CTA's exact DC sums of the job's two
// packed sequences (dc[0] the real part, dc[1] the imaginary part) go to
// dc_out[0..2] and dc_out[3..5] (sum, count, residue in units of 2^-24) the
// same way: a thread's residue sum is a multiple of 2^-24 below 2^-5, so
// r * 2^24 is an exact 32-bit integer and a CTA's total stays below 2^28.
template <int NPOL>
__device__ void commit_stats(const ChainParams& p, const GateStats (&st)[NPOL], uint32_t k, int vals_c,
                       unsigned long long* red, const DcAcc* dc = nullptr, unsigned long long* dc_out = nullptr) {
  constexpr int NS = 4 * NPOL + 4;
  constexpr int NV = NS + 6;
  int v[NV];
  uint32_t n0 = 0, n1 = 0, s0 = 0, s1 = 0;
#pragma unroll
  for (int q = 0; q < NPOL; ++q) {
    v[4 * q + 0] = static_cast<int>(st[q].n0);
    v[4 * q + 1] = static_cast<int>(st[q].n1);
    v[4 * q + 2] = static_cast<int>(st[q].s0);
    v[4 * q + 3] = static_cast<int>(st[q].s1);
    n0 += st[q].n0;
    n1 += st[q].n1;
    s0 += st[q].sat0;
    s1 += st[q].sat1;
  }
  v[4 * NPOL + 0] = static_cast<int>(n0);
  v[4 * NPOL + 1] = static_cast<int>(n1);
  v[4 * NPOL + 2] = static_cast<int>(s0);
  v[4 * NPOL + 3] = static_cast<int>(s1);
  v[NS + 0] = dc ? dc[0].s : 0;
  v[NS + 1] = dc ? dc[0].n : 0;
  v[NS + 2] = dc ? __float2int_rn(dc[0].r * 0x1p24f) : 0;
  v[NS + 3] = dc ? dc[1].s : 0;
  v[NS + 4] = dc ? dc[1].n : 0;
  v[NS + 5] = dc ? __float2int_rn(dc[1].r * 0x1p24f) : 0;
  const int nv = dc_out ? NV : NS;
  int* red32 = reinterpret_cast<int*>(red);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    if (i >= nv) break;
    const int s = __reduce_add_sync(0xffffffffu, v[i]);
    if (lane == 0) red32[warp * NV + i] = s;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    long long tot = 0;
    for (int w = 0; w < nw; ++w) tot += red32[w * NV + threadIdx.x];
    const int i = threadIdx.x;
    if (tot && i >= NS) {
      // DC sums of the job: [0..2] the real part, [3..5] the imaginary part
      atomicAdd(dc_out + (i - NS), static_cast<unsigned long long>(tot));
    } else if (tot) {
      const unsigned long long u = static_cast<unsigned long long>(tot);
      if (i < 4 * NPOL) {
        atomicAdd(p.pol_stats + i, u);
      } else if (i - 4 * NPOL < 2) {
        unsigned long long* cnt =
            reinterpret_cast<unsigned long long*>(p.out + k * p.out_rec + static_cast<uint64_t>(vals_c) * 4);
        atomicAdd(cnt + (i - 4 * NPOL), u);
      } else {
        atomicAdd(p.sat + 2 * k + (i - 4 * NPOL - 2), u);
      }
    }
  }
  __syncthreads();
}


// Row pair rp holds rows rp and N1-rp (rp = 0: rows 0 and N1/2).  Accumulator
// slot a of the pair maps to these bins:
//   rp != 0: a < N2/2 -> row rp, k2 = a (mirror: row N1-rp, N2-1-a);
//            a >= N2/2 -> row N1-rp, k2 = a - N2/2 (mirror: row rp, N2-1-k2)
//   rp == 0: a <= N2/2 -> row 0, k2 = a (mirror: row 0, N2-a mod N2);
//            a > N2/2 -> row N1/2, k2 = a-N2/2-1 (mirror: row N1/2, N2-1-k2)
template <int N2>
__device__ __forceinline__ void pair_slot(uint32_t rp, int a, int& r, int& k2, int& pr, int& k2p) {
  if (rp != 0) {
    if (a < N2 / 2) { r = 0; k2 = a; pr = 1; k2p = N2 - 1 - a; }
    else { r = 1; k2 = a - N2 / 2; pr = 0; k2p = N2 - 1 - k2; }
  } else {
    if (a <= N2 / 2) { r = 0; k2 = a; pr = 0; k2p = (N2 - a) & (N2 - 1); }
    else { r = 1; k2 = a - N2 / 2 - 1; pr = 1; k2p = N2 - 1 - k2; }
  }
}

// Adds one job's contribution to the sums of one bin of a row pair: za is
// Z[k] and zb Z[N-k] of the job's packed complex sequence z = a + i b.
// Power: |A|^2 to a's gate and |B|^2 to b's gate
// (edd/DetectorAccumulator.cuh:40-61); Stokes (dual pol, a = pol 0,
// b = pol 1): I, Q, U, V (edd/src/GatedSpectrometer.cu:125-131) to the job's
// gate.  acc holds [G0, G1] (power) or [I0, I1, Q0, Q1, U0, U1, V0, V1].
template <bool DUAL, int VALS>
__device__ __forceinline__ void accumulate_bin(float (&acc)[VALS], float2 za, float2 zb, uint32_t job) {
  const uint32_t ga = job_ga(job);
  if constexpr (!DUAL) {
    const float sx = za.x + zb.x, sy = za.y - zb.y;
    const float dx = za.x - zb.x, dy = za.y + zb.y;
    const float pa = 0.25f * fmaf(sx, sx, sy * sy);
    const float pb = job_fb(job) != kNoFrame ? 0.25f * fmaf(dx, dx, dy * dy) : 0.f;
    const uint32_t gb = job_gb(job);
    acc[0] += (ga == 0 ? pa : 0.f) + (gb == 0 ? pb : 0.f);
    acc[1] += (ga == 1 ? pa : 0.f) + (gb == 1 ? pb : 0.f);
  } else {
    const float p1x = 0.5f * (za.x + zb.x), p1y = 0.5f * (za.y - zb.y);
    const float p2x = 0.5f * (za.y + zb.y), p2y = -0.5f * (za.x - zb.x);
    const float a1 = fmaf(p1x, p1x, p1y * p1y);
    const float a2 = fmaf(p2x, p2x, p2y * p2y);
    const float I = a1 + a2, Q = a1 - a2;
    const float U = 2.f * fmaf(p1x, p2x, p1y * p2y);
    const float V = -2.f * fmaf(p1y, p2x, -p1x * p2y);
    if (ga == 0) {
      acc[0] += I;
      acc[2] += Q;
      acc[4] += U;
      acc[6] += V;
    } else {
      acc[1] += I;
      acc[3] += Q;
      acc[5] += U;
      acc[7] += V;
    }
  }
}

// Bin 0 of job j of output spectrum k, computed exactly: the real and the
// imaginary packed sequence each sum to (integer in-gate sum) + (residues) +
// (N - in-gate count) * baseline, evaluated in FP64 and rounded once.  An FP32
// FFT forms bin 0 by adding the integer samples and the fractional baseline
// fill in FP32, which rounds with a systematic bias (~1e-5 of the bin at
// 2^20 points); every other bin's rounding is unbiased.
__device__ __forceinline__ float2 exact_dc(const FourStepParams& p, uint32_t k, uint32_t j, uint32_t job,
                                           bool dual) {
  const long long* d = reinterpret_cast<const long long*>(p.dcsum) + (static_cast<size_t>(k) * p.maxjobs + j) * 6;
  const double n = static_cast<double>(p.N1) * static_cast<double>(p.N2);
  const uint32_t ga = job_ga(job);
  const double b_re = p.c.baselines[ga];
  const double b_im = dual ? p.c.baselines[2 + ga] : p.c.baselines[job_gb(job)];
  const double re = static_cast<double>(d[0]) + static_cast<double>(d[2]) * 0x1p-24 +
                    (n - static_cast<double>(d[1])) * b_re;
  const double im = (!dual && job_fb(job) == kNoFrame)
                        ? 0.0
                        : static_cast<double>(d[3]) + static_cast<double>(d[5]) * 0x1p-24 +
                              (n - static_cast<double>(d[4])) * b_im;
  return make_float2(static_cast<float>(re), static_cast<float>(im));
}

// The sums of bin 0 (slot 0 of row pair 0) recomputed from the exact DC of
// every job of output spectrum k, in job order (replacing the FFT's bin 0).
// Every thread of the row-pair-0 CTA calls it (it contains barriers): each
// job's contribution is formed by one thread into `scratch` (at most `cap`
// jobs at a time) and thread 0 adds them into acc0 in job order, which gives
// the same sums as adding the jobs one after the other.
// Stokes I, Q, U, V of one dual-pol job's bin (accumulate_bin without the
// gate selection) added to acc: the caller holds one gate's sums at a time.
__device__ __forceinline__ void accumulate_stokes(float (&acc)[4], float2 za, float2 zb) {
  const float p1x = 0.5f * (za.x + zb.x), p1y = 0.5f * (za.y - zb.y);
  const float p2x = 0.5f * (za.y + zb.y), p2y = -0.5f * (za.x - zb.x);
  const float a1 = fmaf(p1x, p1x, p1y * p1y);
  const float a2 = fmaf(p2x, p2x, p2y * p2y);
  acc[0] += a1 + a2;
  acc[1] += a1 - a2;
  acc[2] += 2.f * fmaf(p1x, p2x, p1y * p2y);
  acc[3] += -2.f * fmaf(p1y, p2x, -p1x * p2y);
}

template <bool DUAL, int VALS>
__device__ __forceinline__ void exact_dc_bin(const FourStepParams& p, uint32_t k, float* scratch, uint32_t cap,
                                             float (&acc0)[VALS]) {
  const uint32_t nj = p.njobs[k];
  const uint32_t tid = threadIdx.x;
  if (tid == 0) {
#pragma unroll
    for (int v = 0; v < VALS; ++v) acc0[v] = 0.f;
  }
  for (uint32_t j0 = 0; j0 < nj; j0 += cap) {
    const uint32_t n = min(cap, nj - j0);
    for (uint32_t t = tid; t < n; t += blockDim.x) {
      float c[VALS];
#pragma unroll
      for (int v = 0; v < VALS; ++v) c[v] = 0.f;
      const uint32_t job = p.jobs[k * p.maxjobs + j0 + t];
      const float2 z = exact_dc(p, k, j0 + t, job, DUAL);
      accumulate_bin<DUAL>(c, z, z, job);
#pragma unroll
      for (int v = 0; v < VALS; ++v) scratch[t * VALS + v] = c[v];
    }
    __syncthreads();
    if (tid == 0)
      for (uint32_t t = 0; t < n; ++t)
#pragma unroll
        for (int v = 0; v < VALS; ++v) acc0[v] += scratch[t * VALS + v];
    __syncthreads();
  }
}

}  // namespace gspec
