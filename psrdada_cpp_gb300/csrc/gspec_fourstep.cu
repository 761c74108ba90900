// Four-step FFT path of the gated spectrometer for N = N1 * N2 >= 8192.
//
// x[N2*n1 + n2] -> pass A: for every column n2 an N1-point FFT over n1
// (unpack + gate fused into the load), times W_N^(n2*k1), stored to scratch
// as Y[k1][n2]; pass B: for every row k1 an N2-point FFT over n2 gives
// Z[k1 + N1*k2].  Rows k1 and N1-k1 hold each bin's mirror N-k, so pass B
// takes them as a pair, splits the packed real sequences and accumulates the
// power (edd/DetectorAccumulator.cuh:40-61) or Stokes
// (edd/src/GatedSpectrometer.cu:140-169) spectra over the jobs of one output
// spectrum, then writes the pair's sums contiguously; the scatter kernel adds
// them into the output record's bins (k1 + N1*k2) with coalesced accesses.
//
// The plan kernel builds each output spectrum's job list (build_jobs): only
// gates holding data are transformed; gates without data add their constant
// baseline to bin 0.
#include "gspec_fourstep_common.cuh"
#include "gspec_kernels.cuh"
#include "gspec_tc_kernels.cuh"

namespace gspec {


// One thread per output spectrum of the launch: its job list (frame order:
// the two gate jobs of a frame are neighbours, so pass A's CTAs that read the
// same frame run close together).
__global__ void fourstep_plan_kernel(FourStepParams p, int dual) {
  const uint32_t kk = blockIdx.x * blockDim.x + threadIdx.x;
  if (kk >= p.nk) return;
  const uint32_t k = p.k0 + kk;
  uint32_t dc[2];
  p.njobs[k] = build_jobs(p.c.flags + k * p.c.nacc, p.c.nacc, dual != 0, p.jobs + k * p.maxjobs, dc);
  p.dc[2 * k] = dc[0];
  p.dc[2 * k + 1] = dc[1];
}

template <int N1>
struct PassACfg {
  static constexpr int BC = N1 >= 1024 ? 8 : 16;     // columns per CTA
  static constexpr int T1 = N1 / 16;
  static constexpr int THREADS = BC * T1;
  static constexpr int STRIDE = spad_size(N1) + 1;  // odd: column-wise reads are conflict-free
  static constexpr size_t RED = static_cast<size_t>(THREADS / 32 > 0 ? THREADS / 32 : 1) * 12 * 8;
  static constexpr size_t TW_BYTES = static_cast<size_t>(tw_size(N1)) * sizeof(float2);
  static constexpr size_t SMEM = static_cast<size_t>(BC) * STRIDE * sizeof(float2) + RED + TW_BYTES;
};

// grid.x = nk * maxjobs * (N2 / BC): (output spectrum, job, column tile)
template <int N1, int NBITS, bool DUAL>
__device__ __forceinline__ void fourstep_a_body(const FourStepParams& p) {
  using Cfg = PassACfg<N1>;
  constexpr int BC = Cfg::BC;
  constexpr int G = Group<NBITS>::samples;
  constexpr int NPOL = DUAL ? 2 : 1;
  extern __shared__ float4 smem_f4[];
  float2* S = reinterpret_cast<float2*>(smem_f4);
  unsigned long long* red =
      reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(smem_f4) + BC * Cfg::STRIDE * sizeof(float2));
  float2* tws = reinterpret_cast<float2*>(reinterpret_cast<char*>(red) + Cfg::RED);

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
  const int tid = threadIdx.x;

  float bl[2 * NPOL];
#pragma unroll
  for (int i = 0; i < 2 * NPOL; ++i) bl[i] = p.c.baselines[i];
  load_twiddles<N1>(tws, p.tw1);

  // spans of SP samples covering this tile's columns of one row: whole
  // groups, or only the tile's part of a group when that part is whole
  // 32-bit words (12-bit samples, 8-column tiles)
  constexpr int SP = (G > BC && (BC * NBITS) % 32 == 0) ? BC : G;
  constexpr int GPR = SP <= BC ? BC / SP : 1;
  const uint32_t gbase = SP <= BC ? c0 : (c0 / SP) * SP;
  const int keep0 = static_cast<int>(c0 - gbase);        // first kept element of a span
  const bool count_stats = (c0 == gbase || SP <= BC);
  const uint32_t sg_a = count_stats ? (DUAL ? (1u << ga) : 3u) : 0u;

  static_assert((N1 * GPR + Cfg::THREADS - 1) / Cfg::THREADS * SP <= 128 && Cfg::THREADS <= 512,
                "per-thread gate statistics fit the 32-bit commit");
  GateStats st[NPOL];
  DcAcc dc[2];
  for (int w = tid; w < N1 * GPR; w += Cfg::THREADS) {
    const int n1 = w % N1;
    const int gi = w / N1;
    const uint32_t gs = gbase + gi * SP;
    const uint32_t off = N2 * n1 + gs;
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
      const int col = static_cast<int>(gs - c0) + e;
      if (SP <= BC || (e >= keep0 && e < keep0 + BC)) S[col * Cfg::STRIDE + spad(n1)] = make_float2(re[e], im[e]);
    }
  }
  // dual pol: the gate statistics leave before the FFT, so they hold no
  // registers there (single pol spills less with them committed at the end)
  if constexpr (DUAL) {
    commit_stats<NPOL>(p.c, st, k, 8 * static_cast<int>(N / 2 + 1), red, dc,
                       p.dcsum + (static_cast<size_t>(k) * p.maxjobs + j) * 6);
  } else {
    __syncthreads();
  }
  {
    const int sq = tid / Cfg::T1;
    const int t = tid - sq * Cfg::T1;
    fft_smem<N1, 16>(S + sq * Cfg::STRIDE, tws, t, true);
  }
  // twiddle W_N^(n2*k1) and store Y[k1][n2].  A thread keeps one column
  // n2 and steps k1 by KS, so W advances by D = W_N^(n2*KS); the exact
  // table value is reloaded every 4th point (at most 3 chained products).
  float2* dst = p.scratch + (static_cast<size_t>(kk) * p.maxjobs + j) * N;
  {
    static_assert(Cfg::THREADS % BC == 0, "a thread keeps one column");
    constexpr int KS = Cfg::THREADS / BC;
    constexpr int PPT = N1 / KS;
    const int col = tid % BC;
    const uint32_t n2 = c0 + col;
    auto exact = [&](uint32_t m) { return cmul(__ldg(&p.twA[m >> 10]), __ldg(&p.twB[m & 1023])); };
    const float2 D = exact(n2 * KS);
    float2 W = make_float2(1.f, 0.f);
#pragma unroll 4
    for (int i = 0; i < PPT; ++i) {
      const int k1 = tid / BC + KS * i;
      W = (i & 3) == 0 ? exact(n2 * static_cast<uint32_t>(k1)) : cmul(W, D);
      const float2 v = S[col * Cfg::STRIDE + spad(k1)];
      dst[static_cast<size_t>(k1) * N2 + n2] = cmul(v, W);
    }
  }
  if constexpr (!DUAL)
    commit_stats<NPOL>(p.c, st, k, 2 * static_cast<int>(N / 2 + 1), red, dc,
                       p.dcsum + (static_cast<size_t>(k) * p.maxjobs + j) * 6);
}

// Columns of up to 256 points (at most 256 threads) are held to 64 registers
// so that 65536 / (THREADS * 64) CTAs share an SM (4 at 256 points).
template <int N1>
constexpr int pass_a_min_blocks() {
  return PassACfg<N1>::THREADS <= 256 ? 65536 / (PassACfg<N1>::THREADS * 64) : 1;
}
template <int N1, int NBITS, bool DUAL>
__global__ void __launch_bounds__(PassACfg<N1>::THREADS, pass_a_min_blocks<N1>()) fourstep_a_kernel(FourStepParams p) {
  fourstep_a_body<N1, NBITS, DUAL>(p);
}

// The same pass held to 64 registers so that two 512-thread CTAs share an SM.
#ifndef GSPEC_PASSA_2CTA
#define GSPEC_PASSA_2CTA 1
#endif
template <int N1, int NBITS, bool DUAL>
__global__ void __launch_bounds__(PassACfg<N1>::THREADS, 2) fourstep_a_2cta_kernel(FourStepParams p) {
  fourstep_a_body<N1, NBITS, DUAL>(p);
}

#ifndef GSPEC_PASSB_THREADS
#define GSPEC_PASSB_THREADS 0   // 0: 256 threads for rows of up to 512 points, 128 for 1024
#endif
#ifndef GSPEC_PASSB_STAGES
#define GSPEC_PASSB_STAGES 2
#endif
#ifndef GSPEC_PASSB_MINB
#define GSPEC_PASSB_MINB 2   // resident CTAs per SM the register allocation is sized for
#endif

template <int N2, bool DUAL>
struct PassBCfg {
  // 256 threads at N2 = 256 run pass B 7 % faster than 128 (16 warps per SM
  // instead of 12, 117 registers); at N2 = 1024 they would spill the
  // per-thread bin sums (9 x 8 floats at 128 threads) and run 8 % slower
  static constexpr int BASE = GSPEC_PASSB_THREADS > 0 ? GSPEC_PASSB_THREADS : (N2 >= 1024 ? 128 : 256);
  static constexpr int THREADS = BASE >= 2 * (N2 / 16) ? BASE : 2 * (N2 / 16);
  static constexpr int T2 = N2 / 16;
  static constexpr int JOB_THREADS = 2 * T2;         // one job: rows rp and N1-rp
  static constexpr int J = THREADS / JOB_THREADS;    // jobs transformed together
  static constexpr int STRIDE = spad_size(N2);
  static constexpr int VALS = DUAL ? 8 : 2;
  // dual pol at 1024-point rows: the CTA visits the spectrum's gate-0 jobs,
  // then its gate-1 jobs (a permutation in shared memory), so a thread holds
  // one gate's I, Q, U, V per bin at a time: half the bin sums, 157 instead
  // of 204 registers, three CTAs per SM
  static constexpr bool BANK = DUAL && N2 == 1024;
  static constexpr int HELD = BANK ? 4 : VALS;   // values a thread sums per bin at a time
  static constexpr int BPT = (N2 + 1 + THREADS - 1) / THREADS;   // output bins per thread
  static constexpr int STAGE_F2 = J * 2 * N2;        // one TMA stage: J jobs x 2 rows, unpadded
  static constexpr size_t STAGE_BYTES = static_cast<size_t>(STAGE_F2) * sizeof(float2);
  static constexpr size_t WORK_BYTES = static_cast<size_t>(2 * J) * STRIDE * sizeof(float2);
  static constexpr size_t TW_BYTES = static_cast<size_t>(tw_size(N2)) * sizeof(float2);
  static constexpr size_t JW_BYTES = ((J * sizeof(uint32_t)) + 15) / 16 * 16;
  static constexpr int NST = GSPEC_PASSB_STAGES;     // TMA stages: NST - 1 groups ahead
  static constexpr size_t SMEM = NST * STAGE_BYTES + WORK_BYTES + TW_BYTES + JW_BYTES + NST * sizeof(uint64_t);
  // resident CTAs the register allocation is sized for
  static constexpr int MINB = BANK ? 3 : GSPEC_PASSB_MINB;
};


// grid.x = nk * N1/2: unit (output spectrum k, row pair rp).  J jobs are
// transformed together (2*T2 threads each).  Their rows arrive by TMA bulk
// copies into one of NST staging buffers, NST - 1 groups ahead of the group
// being transformed; the first FFT pass reads the staging buffer.  Thread t owns
// output slots a = t + THREADS*i of the pair and keeps their power / Stokes
// sums in registers over all jobs of the spectrum, adding the jobs in
// order, so the result does not depend on scheduling.
template <int N2, bool DUAL>
__global__ void __launch_bounds__(PassBCfg<N2, DUAL>::THREADS, PassBCfg<N2, DUAL>::MINB) fourstep_b_kernel(FourStepParams p) {
  using Cfg = PassBCfg<N2, DUAL>;
  constexpr int J = Cfg::J;
  constexpr int BPT = Cfg::BPT;
  constexpr int VALS = Cfg::VALS;
  constexpr int NST = Cfg::NST;
  constexpr uint32_t kRowBytes = N2 * sizeof(float2);
  extern __shared__ float4 smem_f4[];
  char* base = reinterpret_cast<char*>(smem_f4);
  float2* stage = reinterpret_cast<float2*>(base);                           // [NST][J][2][N2]
  float2* work = reinterpret_cast<float2*>(base + NST * Cfg::STAGE_BYTES);   // [J][2][STRIDE]
  float2* tws = reinterpret_cast<float2*>(base + NST * Cfg::STAGE_BYTES + Cfg::WORK_BYTES);
  uint32_t* jw = reinterpret_cast<uint32_t*>(base + NST * Cfg::STAGE_BYTES + Cfg::WORK_BYTES + Cfg::TW_BYTES);
  uint64_t* bar = reinterpret_cast<uint64_t*>(base + NST * Cfg::STAGE_BYTES + Cfg::WORK_BYTES + Cfg::TW_BYTES +
                                              Cfg::JW_BYTES);

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
  const int q = tid / Cfg::JOB_THREADS;            // job of this thread during the FFT
  const int lt = tid - q * Cfg::JOB_THREADS;

  const uint32_t njobs = p.njobs[k];
  const uint32_t* jobs = p.jobs + k * p.maxjobs;
  const uint32_t ngroups = (njobs + J - 1) / J;
  // BANK: the spectrum's job words and the visiting order (gate-0 jobs, then
  // gate-1 jobs, each in list order) after the barriers, [maxjobs] each
  uint32_t* words = reinterpret_cast<uint32_t*>(bar + NST);
  uint32_t* order = words + p.maxjobs;
  if constexpr (Cfg::BANK) {
    for (uint32_t i = tid; i < njobs; i += Cfg::THREADS) words[i] = jobs[i];
    __syncthreads();
  }
  if (tid == 0) {
#pragma unroll
    for (int i = 0; i < NST; ++i) mbar_init(&bar[i], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    if constexpr (Cfg::BANK) {
      uint32_t w = 0;
      for (uint32_t i = 0; i < njobs; ++i)
        if (job_ga(words[i]) == 0) order[w++] = i;
      for (uint32_t i = 0; i < njobs; ++i)
        if (job_ga(words[i]) != 0) order[w++] = i;
    }
  }
  // list position of the i-th job this CTA visits
  auto slot_of = [&](uint32_t i) -> uint32_t {
    if constexpr (Cfg::BANK) return order[i];
    else return i;
  };
  load_twiddles<N2>(tws, p.tw2);
  __syncthreads();
  // thread 0: rows of job group g into stage s
  auto issue = [&](uint32_t g, int s) {
    const uint32_t nq = min(static_cast<uint32_t>(J), njobs - g * J);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    mbar_expect_tx(&bar[s], nq * 2 * kRowBytes);
    for (uint32_t qq = 0; qq < nq; ++qq) {
      const float2* seq = p.scratch + (static_cast<size_t>(kk) * p.maxjobs + slot_of(g * J + qq)) * N;
      float2* dst = stage + static_cast<size_t>(s) * Cfg::STAGE_F2 + qq * 2 * N2;
      bulk_g2s(dst, seq + static_cast<size_t>(rowA) * N2, kRowBytes, &bar[s]);
      bulk_g2s(dst + N2, seq + static_cast<size_t>(rowB) * N2, kRowBytes, &bar[s]);
    }
  };
  if (tid == 0)
    for (uint32_t g = 0; g + 1 < static_cast<uint32_t>(NST) && g < ngroups; ++g) issue(g, static_cast<int>(g));

  // job words one group ahead: the global load of group g + 1 is in flight
  // while group g is transformed
  auto job_at = [&](uint32_t i) -> uint32_t {
    if constexpr (Cfg::BANK) return words[order[i]];
    else return jobs[i];
  };
  uint32_t next_job = (tid < J && static_cast<uint32_t>(tid) < njobs) ? job_at(tid) : 0u;
  constexpr int HELD = Cfg::HELD;
  float acc[BPT][HELD];
#pragma unroll
  for (int i = 0; i < BPT; ++i)
#pragma unroll
    for (int v = 0; v < HELD; ++v) acc[i][v] = 0.f;
  // row-pair sums, contiguous in the slot a (coalesced); fourstep_scatter_kernel
  // moves them into the output bins, whose index c strides by N1 along a.
  // Value v of slot a at bs[v * (N2 + 1) + a]; dual pol: v = 2 * stokes + gate.
  float* bs = p.bsum + static_cast<size_t>(blockIdx.x) * VALS * (N2 + 1);
  uint32_t cur = 0;   // BANK: the gate whose sums acc holds

  for (uint32_t g = 0; g < ngroups; ++g) {
    const int s = static_cast<int>(g % NST);
    // the stage of group g + NST - 1 held group g - 1, done at the last barrier
    if (tid == 0 && g + NST - 1 < ngroups) issue(g + NST - 1, static_cast<int>((g + NST - 1) % NST));
    const bool ok = mbar_wait(&bar[s], (g / NST) & 1u, 1u << 24);
    if (__syncthreads_or(!ok)) {
      if (tid == 0) {
        if (p.c.dev_err) atomicExch(p.c.dev_err, 2u);
        // give the copies still in flight a bounded chance to land before exit
        for (uint32_t h = g; h < g + NST && h < ngroups; ++h)
          mbar_wait(&bar[h % NST], (h / NST) & 1u, 1u << 20);
      }
      __syncthreads();
      break;
    }
    const uint32_t j0 = g * J;
    const int nq = static_cast<int>(min(static_cast<uint32_t>(J), njobs - j0));
    const bool active = q < nq;
    if (tid < nq) jw[tid] = next_job;
    if (tid < J && j0 + J + tid < njobs) next_job = job_at(j0 + J + tid);
    {
      const int r = lt / Cfg::T2;
      const int t = lt - r * Cfg::T2;
      fft_smem_from<N2, 16>(stage + static_cast<size_t>(s) * Cfg::STAGE_F2 + (q * 2 + r) * N2,
                            work + (2 * q + r) * Cfg::STRIDE, tws, t, active);
    }
    // BANK: the group's first job of gate 1, where gate 0's sums are complete
    int qb = nq;
    if constexpr (Cfg::BANK) {
      if (cur == 0)
        for (int qq = 0; qq < nq; ++qq)
          if (job_ga(jw[qq]) != 0) {
            qb = qq;
            break;
          }
    }
#pragma unroll
    for (int i = 0; i < BPT; ++i) {
      const int a = tid + i * Cfg::THREADS;
      if (a >= nbins) continue;
      int r, k2, pr, k2p;
      pair_slot<N2>(rp, a, r, k2, pr, k2p);
      for (int qq = 0; qq < nq; ++qq) {
        const uint32_t job = jw[qq];
        const float2 za = work[(2 * qq + r) * Cfg::STRIDE + spad(k2)];
        const float2 zb = work[(2 * qq + pr) * Cfg::STRIDE + spad(k2p)];
        if constexpr (Cfg::BANK) {
          if (qq == qb) {
#pragma unroll
            for (int v = 0; v < 4; ++v) {
              bs[(2 * v) * (N2 + 1) + a] = acc[i][v];
              acc[i][v] = 0.f;
            }
          }
          accumulate_stokes(acc[i], za, zb);
        } else {
          accumulate_bin<DUAL>(acc[i], za, zb, job);
        }
      }
    }
    if (Cfg::BANK && qb < nq) cur = 1;
    __syncthreads();
  }
  // the sums held at the end (BANK: gate `cur`; a gate without jobs sums to 0)
#pragma unroll
  for (int i = 0; i < BPT; ++i) {
    const int a = tid + i * Cfg::THREADS;
    if (a >= nbins) continue;
    if constexpr (Cfg::BANK) {
#pragma unroll
      for (int v = 0; v < 4; ++v) {
        bs[(2 * v + cur) * (N2 + 1) + a] = acc[i][v];
        if (cur == 0) bs[(2 * v + 1) * (N2 + 1) + a] = 0.f;
      }
    } else {
#pragma unroll
      for (int v = 0; v < VALS; ++v) bs[v * (N2 + 1) + a] = acc[i][v];
    }
  }
  (void)C;
  // bin 0 (row pair 0, slot 0, thread 0) from the exact per-job sums
  // (exact_dc), over the jobs in order, plus the constant baseline of gates
  // without data; the work buffer is free after the loop's last barrier
  if (rp == 0) {
    float c0[VALS];
    exact_dc_bin<DUAL>(p, k, reinterpret_cast<float*>(work),
                       static_cast<uint32_t>(Cfg::WORK_BYTES / (VALS * sizeof(float))), c0);
    if (tid == 0) {
      const float n = static_cast<float>(N);
      for (int gate = 0; gate < 2; ++gate) {
        const float cnt = static_cast<float>(p.dc[2 * k + gate]);
        if (cnt == 0.f) continue;
        if constexpr (!DUAL) {
          const float d = n * p.c.baselines[gate];
          c0[gate] += cnt * d * d;
        } else {
          const float x = n * p.c.baselines[gate], y = n * p.c.baselines[2 + gate];
          c0[0 + gate] += cnt * (x * x + y * y);
          c0[2 + gate] += cnt * (x * x - y * y);
          c0[4 + gate] += cnt * (2.f * x * y);
        }
      }
#pragma unroll
      for (int v = 0; v < VALS; ++v) bs[v * (N2 + 1)] = c0[v];
    }
  }
}

// Adds the row-pair sums of one launch into the output spectra.  Output bin
// c = k1 + N1*k2 sits in row pair rp at slot a (the inverse of pair_slot):
//   k1 = 0: rp 0, a = k2; k1 = N1/2: rp 0, a = N2/2 + 1 + k2;
//   k1 < N1/2: rp = k1, a = k2; else rp = N1 - k1, a = N2/2 + k2.
// Along k2 the slots are contiguous, along k1 the bins are, so a CTA moves a
// 32 x 32 tile of (k1, k2) through shared memory: it reads 32 slots of each
// of its 32 row pairs and writes 32 consecutive bins of each of its 32 k2
// rows, both as 128-byte runs.  With store set (the launch holds every
// contribution to its spectra, so the caller's zeroed bins would only be
// read back) the bins are written instead of read, added and written.
// grid = (N1 / 32, ceil((N2/2 + 1) / 32), nk * VALS), block = (32, 8).
__global__ void __launch_bounds__(256) fourstep_scatter_kernel(FourStepParams p, int vals, int store) {
  __shared__ float tile[32][33];
  const uint32_t N1 = p.N1, N2 = p.N2;
  const uint32_t C = N1 * N2 / 2 + 1;
  const uint32_t kk = blockIdx.z / vals;
  const uint32_t v = blockIdx.z - kk * vals;
  const uint32_t k1_0 = blockIdx.x * 32, k2_0 = blockIdx.y * 32;
  const uint32_t lane = threadIdx.x;
  const size_t rp_stride = static_cast<size_t>(vals) * (N2 + 1);
  const float* bs = p.bsum + (static_cast<size_t>(kk) * (N1 / 2) * vals + v) * (N2 + 1);
#pragma unroll
  for (uint32_t i = threadIdx.y; i < 32; i += 8) {
    const uint32_t k1 = k1_0 + i, k2 = k2_0 + lane;
    if (k1 + N1 * k2 >= C) continue;
    uint32_t rp, a;
    if (k1 == 0) {
      rp = 0;
      a = k2;
    } else if (k1 == N1 / 2) {
      rp = 0;
      a = N2 / 2 + 1 + k2;
    } else if (k1 < N1 / 2) {
      rp = k1;
      a = k2;
    } else {
      rp = N1 - k1;
      a = N2 / 2 + k2;
    }
    tile[i][lane] = bs[rp * rp_stride + a];
  }
  __syncthreads();
  float* outf = reinterpret_cast<float*>(p.c.out + (p.k0 + kk) * p.c.out_rec) + static_cast<size_t>(v) * C;
#pragma unroll
  for (uint32_t i = threadIdx.y; i < 32; i += 8) {
    const uint32_t c = k1_0 + lane + N1 * (k2_0 + i);
    if (c >= C) continue;
    const float x = tile[lane][i];
    outf[c] = store ? x : outf[c] + x;
  }
}

// ------------------------------------------------------------ dispatch
int fourstep_n1(int N) {
  int L = 0;
  while ((1 << L) < N) ++L;
  int L1 = L / 2;
  if (L1 > 10) L1 = 10;
  return 1 << L1;
}
int fourstep_n2(int N) { return N / fourstep_n1(N); }
bool fourstep_supported(int N) {
  if (N < 8192 || N > (1 << 20) || (N & (N - 1))) return false;
  const int n2 = fourstep_n2(N);
  return n2 >= 128 && n2 <= 1024;
}

template <int N1, bool DUAL>
static cudaError_t launch_a_n1(int nbits, const FourStepParams& p, cudaStream_t s) {
  using Cfg = PassACfg<N1>;
  const unsigned grid = p.nk * p.maxjobs * (p.N2 / Cfg::BC);
  auto run = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(Cfg::SMEM));
    if (e != cudaSuccess) return e;
    kern<<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(p);
    return cudaGetLastError();
  };
  // 1024-point columns (512 threads) at 78 registers leave one CTA per SM;
  // held to 64 they fit two (8- and 12-bit; 10-bit, and 512-point columns,
  // would spill)
  if constexpr (GSPEC_PASSA_2CTA && N1 == 1024) {
    switch (nbits) {
      case 8: return run(fourstep_a_2cta_kernel<N1, 8, DUAL>);
      case 10: return run(fourstep_a_kernel<N1, 10, DUAL>);
      case 12: return run(fourstep_a_2cta_kernel<N1, 12, DUAL>);
    }
  } else {
    switch (nbits) {
      case 8: return run(fourstep_a_kernel<N1, 8, DUAL>);
      case 10: return run(fourstep_a_kernel<N1, 10, DUAL>);
      case 12: return run(fourstep_a_kernel<N1, 12, DUAL>);
    }
  }
  return cudaErrorInvalidValue;
}

template <int N2, bool DUAL>
static cudaError_t launch_b_n2(const FourStepParams& p, cudaStream_t s) {
  using Cfg = PassBCfg<N2, DUAL>;
  const unsigned grid = p.nk * (p.N1 / 2);
  const size_t smem = Cfg::SMEM + (Cfg::BANK ? 2 * static_cast<size_t>(p.maxjobs) * sizeof(uint32_t) : 0);
  auto kern = fourstep_b_kernel<N2, DUAL>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  if (e != cudaSuccess) return e;
  kern<<<grid, Cfg::THREADS, smem, s>>>(p);
  return cudaGetLastError();
}

template <bool DUAL>
static cudaError_t launch_fs(int nbits, const FourStepParams& p, int pass, cudaStream_t s) {
  if (pass == 0) {
    switch (p.N1) {
      case 64: return launch_a_n1<64, DUAL>(nbits, p, s);
      case 128: return launch_a_n1<128, DUAL>(nbits, p, s);
      case 256: return launch_a_n1<256, DUAL>(nbits, p, s);
      case 512: return launch_a_n1<512, DUAL>(nbits, p, s);
      case 1024: return launch_a_n1<1024, DUAL>(nbits, p, s);
    }
    return cudaErrorInvalidValue;
  }
  switch (p.N2) {
    case 128: return launch_b_n2<128, DUAL>(p, s);
    case 256: return launch_b_n2<256, DUAL>(p, s);
    case 512: return launch_b_n2<512, DUAL>(p, s);
    case 1024: return launch_b_n2<1024, DUAL>(p, s);
  }
  return cudaErrorInvalidValue;
}

// pass: -1 plan, 0 pass A, 1 pass B, 2 scatter of the pass-B sums
cudaError_t launch_fourstep(int N, int nbits, bool dual, const FourStepParams& p, int pass, cudaStream_t s) {
  (void)N;
  if (pass < 0) {
    fourstep_plan_kernel<<<(p.nk + 63) / 64, 64, 0, s>>>(p, dual ? 1 : 0);
    return cudaGetLastError();
  }
  if (pass == 2) {
    const int vals = dual ? 8 : 2;
    fourstep_scatter_kernel<<<dim3(p.N1 / 32, (p.N2 / 2 + 1 + 31) / 32, p.nk * vals), dim3(32, 8), 0, s>>>(
        p, vals, p.c.store ? 1 : 0);
    return cudaGetLastError();
  }
  if (p.form != 0 && ((pass == 0 && p.N1 == 1024) || (pass == 1 && p.N2 == 1024)))
    return tc::launch_tc_pass(pass, nbits, dual, p, s);
  return dual ? launch_fs<true>(nbits, p, pass, s) : launch_fs<false>(nbits, p, pass, s);
}

}  // namespace gspec
