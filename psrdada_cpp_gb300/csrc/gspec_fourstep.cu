// Four-step FFT path of the gated spectrometer for N = N1 * N2 >= 8192.
//
// x[N2*n1 + n2] -> pass A: for every column n2 an N1-point FFT over n1
// (unpack + gate fused into the load), times W_N^(n2*k1), stored to scratch
// as Y[k1][n2]; pass B: for every row k1 an N2-point FFT over n2 gives
// Z[k1 + N1*k2].  Rows k1 and N1-k1 hold each bin's mirror N-k, so pass B
// takes them as a pair, splits the packed real sequences and accumulates the
// power (edd/DetectorAccumulator.cuh:40-61) or Stokes
// (edd/src/GatedSpectrometer.cu:140-169) spectra over the frames of one
// output spectrum before writing them once.
//
// Pass A runs once per gate: single pol packs G0 + i G1 (one sequence);
// dual pol packs P0 + i P1 of gate 0 or gate 1 (grid dimension).
#include "gspec_kernels.cuh"

namespace gspec {

namespace {

__device__ __forceinline__ unsigned long long warp_sum(unsigned long long v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// Same commit rule as the small path: per-pol n0, n1, s0, s1 to pol_stats;
// n0, n1 summed over pols to the output record; saturation to sat[k].
template <int NPOL>
__device__ void commit(const ChainParams& p, const GateStats (&st)[NPOL], uint32_t k, int vals_c,
                       unsigned long long* red) {
  constexpr int NV = 4 * NPOL + 4;
  unsigned long long v[NV];
  unsigned long long n0 = 0, n1 = 0, s0 = 0, s1 = 0;
#pragma unroll
  for (int q = 0; q < NPOL; ++q) {
    v[4 * q + 0] = st[q].n0;
    v[4 * q + 1] = st[q].n1;
    v[4 * q + 2] = static_cast<unsigned long long>(st[q].s0);
    v[4 * q + 3] = static_cast<unsigned long long>(st[q].s1);
    n0 += st[q].n0;
    n1 += st[q].n1;
    s0 += st[q].sat0;
    s1 += st[q].sat1;
  }
  v[4 * NPOL + 0] = n0;
  v[4 * NPOL + 1] = n1;
  v[4 * NPOL + 2] = s0;
  v[4 * NPOL + 3] = s1;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int i = 0; i < NV; ++i) {
    unsigned long long s = warp_sum(v[i]);
    if (lane == 0) red[warp * NV + i] = s;
  }
  __syncthreads();
  if (threadIdx.x < NV) {
    unsigned long long tot = 0;
    for (int w = 0; w < nw; ++w) tot += red[w * NV + threadIdx.x];
    const int i = threadIdx.x;
    if (tot) {
      if (i < 4 * NPOL) {
        atomicAdd(p.pol_stats + i, tot);
      } else if (i - 4 * NPOL < 2) {
        unsigned long long* cnt =
            reinterpret_cast<unsigned long long*>(p.out + k * p.out_rec + static_cast<uint64_t>(vals_c) * 4);
        atomicAdd(cnt + (i - 4 * NPOL), tot);
      } else {
        atomicAdd(p.sat + 2 * k + (i - 4 * NPOL - 2), tot);
      }
    }
  }
  __syncthreads();
}

}  // namespace

template <int N1>
struct PassACfg {
  static constexpr int BC = N1 >= 1024 ? 8 : 16;     // columns per CTA
  static constexpr int T1 = N1 / 16;
  static constexpr int THREADS = BC * T1;
  static constexpr int STRIDE = spad_size(N1) + 1;  // odd: column-wise reads are conflict-free
  static constexpr size_t RED = static_cast<size_t>(THREADS / 32) * 12 * 8;
  static constexpr size_t SMEM = static_cast<size_t>(BC) * STRIDE * sizeof(float2) + RED;
};

// grid.x = nframes * (N2 / BC) * ngates
template <int N1, int NBITS, bool DUAL>
__global__ void __launch_bounds__(PassACfg<N1>::THREADS) fourstep_a_kernel(FourStepParams p) {
  using Cfg = PassACfg<N1>;
  constexpr int BC = Cfg::BC;
  constexpr int G = Group<NBITS>::samples;
  constexpr int NPOL = DUAL ? 2 : 1;
  constexpr int NGATES = DUAL ? 2 : 1;
  extern __shared__ float4 smem_f4[];
  float2* S = reinterpret_cast<float2*>(smem_f4);
  unsigned long long* red =
      reinterpret_cast<unsigned long long*>(reinterpret_cast<char*>(smem_f4) + BC * Cfg::STRIDE * sizeof(float2));

  const uint32_t N2 = p.N2;
  const uint32_t N = N1 * N2;
  const uint32_t tiles = N2 / BC;
  uint32_t u = blockIdx.x;
  const uint32_t gate = u % NGATES;
  u /= NGATES;
  const uint32_t tile = u % tiles;
  const uint32_t fl = u / tiles;
  const uint32_t f = p.frame0 + fl;
  const uint32_t k = f / p.c.nacc;
  const uint32_t c0 = tile * BC;
  const int tid = threadIdx.x;

  float bl[2 * NPOL];
#pragma unroll
  for (int i = 0; i < 2 * NPOL; ++i) bl[i] = p.c.baselines[i];

  // groups covering this tile's columns of one row
  constexpr int GPR = G <= BC ? BC / G : 1;
  const uint32_t gbase = G <= BC ? c0 : (c0 / G) * G;
  const int keep0 = static_cast<int>(c0 - gbase);        // first kept element of a group
  const bool count_stats = (gate == 0) && (c0 == gbase || G <= BC);

  GateStats st[NPOL];
  GateStats junk[NPOL];
  for (int w = tid; w < N1 * GPR; w += Cfg::THREADS) {
    const int n1 = w % N1;
    const int gi = w / N1;
    const uint32_t gs = gbase + gi * G;
    const uint32_t s = f * N + N2 * n1 + gs;
    float a0[G], a1[G];
    gate_group<NBITS>(p.c.g, 0, s, bl[0], bl[1], a0, a1, count_stats ? st[0] : junk[0]);
    float b0[G], b1[G];
    if constexpr (DUAL) {
      gate_group<NBITS>(p.c.g, 1, s, bl[2], bl[3], b0, b1, count_stats ? st[NPOL - 1] : junk[NPOL - 1]);
    }
#pragma unroll
    for (int e = 0; e < G; ++e) {
      const int col = static_cast<int>(gs - c0) + e;
      if (G <= BC || (e >= keep0 && e < keep0 + BC)) {
        float2 z;
        if constexpr (DUAL) {
          z = gate ? make_float2(a1[e], b1[e]) : make_float2(a0[e], b0[e]);
        } else {
          z = make_float2(a0[e], a1[e]);
        }
        S[col * Cfg::STRIDE + spad(n1)] = z;
      }
    }
  }
  __syncthreads();
  {
    const int sq = tid / Cfg::T1;
    const int t = tid - sq * Cfg::T1;
    fft_smem<N1, 16>(S + sq * Cfg::STRIDE, p.tw1, t, true);
  }
  // twiddle W_N^(n2*k1) and store Y[k1][n2]
  float2* dst = p.scratch + (static_cast<size_t>(fl) * NGATES + gate) * N;
  for (int w = tid; w < BC * N1; w += Cfg::THREADS) {
    const int col = w % BC;
    const int k1 = w / BC;
    float2 v = S[col * Cfg::STRIDE + spad(k1)];
    const uint32_t m = (c0 + col) * static_cast<uint32_t>(k1);
    const float2 W = cmul(__ldg(&p.twA[m >> 10]), __ldg(&p.twB[m & 1023]));
    dst[static_cast<size_t>(k1) * N2 + c0 + col] = cmul(v, W);
  }
  if (gate == 0) commit<NPOL>(p.c, st, k, (DUAL ? 8 : 2) * static_cast<int>(N / 2 + 1), red);
}

template <int N2, bool DUAL>
struct PassBCfg {
  static constexpr int SEQ = DUAL ? 2 : 1;
  static constexpr int T2 = N2 / 16;
  static constexpr int THREADS = 2 * SEQ * T2;
  static constexpr int STRIDE = spad_size(N2);
  static constexpr int VALS = DUAL ? 8 : 2;
  static constexpr int NA = N2 + 1;                  // accumulated bins per row pair
  static constexpr size_t SMEM =
      static_cast<size_t>(2 * SEQ) * STRIDE * sizeof(float2) + static_cast<size_t>(VALS) * NA * sizeof(float);
};

// grid.x = nk * N1/2: unit (output spectrum k, row pair rp)
template <int N2, bool DUAL>
__global__ void __launch_bounds__(PassBCfg<N2, DUAL>::THREADS) fourstep_b_kernel(FourStepParams p) {
  using Cfg = PassBCfg<N2, DUAL>;
  constexpr int SEQ = Cfg::SEQ;
  constexpr int NA = Cfg::NA;
  extern __shared__ float4 smem_f4[];
  float2* S = reinterpret_cast<float2*>(smem_f4);      // [row r][seq] sequences
  float* acc = reinterpret_cast<float*>(S + 2 * SEQ * Cfg::STRIDE);

  const uint32_t N1 = p.N1;
  const uint32_t N = N1 * N2;
  const uint32_t C = N / 2 + 1;
  const uint32_t half = N1 / 2;
  const uint32_t k = p.k0 + blockIdx.x / half;
  const uint32_t rp = blockIdx.x % half;
  const uint32_t rowA = rp;
  const uint32_t rowB = rp == 0 ? half : N1 - rp;
  const int tid = threadIdx.x;

  for (int i = tid; i < Cfg::VALS * NA; i += Cfg::THREADS) acc[i] = 0.f;

  const int nbins = rp == 0 ? N2 + 1 : N2;
  for (uint32_t fr = 0; fr < p.c.nacc; ++fr) {
    const uint32_t fl = k * p.c.nacc + fr - p.frame0;
#pragma unroll
    for (int r = 0; r < 2; ++r) {
#pragma unroll
      for (int sq = 0; sq < SEQ; ++sq) {
        const float4* src = reinterpret_cast<const float4*>(
            p.scratch + ((static_cast<size_t>(fl) * SEQ + sq) * N1 + (r ? rowB : rowA)) * N2);
        float2* d = S + (r * SEQ + sq) * Cfg::STRIDE;
        for (int i = tid; i < N2 / 2; i += Cfg::THREADS) {
          const float4 q = src[i];
          d[spad(2 * i)] = make_float2(q.x, q.y);
          d[spad(2 * i + 1)] = make_float2(q.z, q.w);
        }
      }
    }
    __syncthreads();
    {
      const int sq = tid / Cfg::T2;
      const int t = tid - sq * Cfg::T2;
      fft_smem<N2, 16>(S + sq * Cfg::STRIDE, p.tw2, t, true);
    }
    for (int a = tid; a < nbins; a += Cfg::THREADS) {
      int r, k2, pr, k2p;
      if (rp != 0) {
        if (a < N2 / 2) { r = 0; k2 = a; pr = 1; k2p = N2 - 1 - a; }
        else { r = 1; k2 = a - N2 / 2; pr = 0; k2p = N2 - 1 - k2; }
      } else {
        if (a <= N2 / 2) { r = 0; k2 = a; pr = 0; k2p = (N2 - a) & (N2 - 1); }
        else { r = 1; k2 = a - N2 / 2 - 1; pr = 1; k2p = N2 - 1 - k2; }
      }
#pragma unroll
      for (int sq = 0; sq < SEQ; ++sq) {
        const float2 za = S[(r * SEQ + sq) * Cfg::STRIDE + spad(k2)];
        const float2 zb = S[(pr * SEQ + sq) * Cfg::STRIDE + spad(k2p)];
        if constexpr (!DUAL) {
          const float sx = za.x + zb.x, sy = za.y - zb.y;
          const float dx = za.x - zb.x, dy = za.y + zb.y;
          acc[a] += 0.25f * fmaf(sx, sx, sy * sy);
          acc[NA + a] += 0.25f * fmaf(dx, dx, dy * dy);
        } else {
          const float p1x = 0.5f * (za.x + zb.x), p1y = 0.5f * (za.y - zb.y);
          const float p2x = 0.5f * (za.y + zb.y), p2y = -0.5f * (za.x - zb.x);
          const float a1 = fmaf(p1x, p1x, p1y * p1y);
          const float a2 = fmaf(p2x, p2x, p2y * p2y);
          acc[(0 + sq) * NA + a] += a1 + a2;
          acc[(2 + sq) * NA + a] += a1 - a2;
          acc[(4 + sq) * NA + a] += 2.f * fmaf(p1x, p2x, p1y * p2y);
          acc[(6 + sq) * NA + a] += -2.f * fmaf(p1y, p2x, -p1x * p2y);
        }
      }
    }
    __syncthreads();
  }
  float* outf = reinterpret_cast<float*>(p.c.out + k * p.c.out_rec);
  for (int i = tid; i < Cfg::VALS * nbins; i += Cfg::THREADS) {
    const int v = i / nbins;
    const int a = i - v * nbins;
    uint32_t c;
    if (rp != 0) {
      c = a < N2 / 2 ? rp + N1 * a : (N1 - rp) + N1 * (a - N2 / 2);
    } else {
      c = a <= N2 / 2 ? N1 * a : half + N1 * (a - N2 / 2 - 1);
    }
    outf[static_cast<size_t>(v) * C + c] += acc[v * NA + a];
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
  const unsigned grid = p.nframes * (p.N2 / Cfg::BC) * (DUAL ? 2 : 1);
  auto run = [&](auto kern) -> cudaError_t {
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(Cfg::SMEM));
    if (e != cudaSuccess) return e;
    kern<<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(p);
    return cudaGetLastError();
  };
  switch (nbits) {
    case 8: return run(fourstep_a_kernel<N1, 8, DUAL>);
    case 10: return run(fourstep_a_kernel<N1, 10, DUAL>);
    case 12: return run(fourstep_a_kernel<N1, 12, DUAL>);
  }
  return cudaErrorInvalidValue;
}

template <int N2, bool DUAL>
static cudaError_t launch_b_n2(const FourStepParams& p, cudaStream_t s) {
  using Cfg = PassBCfg<N2, DUAL>;
  const unsigned grid = p.nk * (p.N1 / 2);
  auto kern = fourstep_b_kernel<N2, DUAL>;
  cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(Cfg::SMEM));
  if (e != cudaSuccess) return e;
  kern<<<grid, Cfg::THREADS, Cfg::SMEM, s>>>(p);
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

cudaError_t launch_fourstep(int N, int nbits, bool dual, const FourStepParams& p, int pass, cudaStream_t s) {
  (void)N;
  return dual ? launch_fs<true>(nbits, p, pass, s) : launch_fs<false>(nbits, p, pass, s);
}

}  // namespace gspec
