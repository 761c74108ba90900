// Kernel parameter blocks and launch helpers shared by the kernels and the
// host engine.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include "gspec_device.cuh"

namespace gspec {

// Per-pol statistics of the block being processed (reset by finalize):
// [pol][0] n0, [1] n1, [2] sum0 (two's complement), [3] sum1.
constexpr int kPolStats = 4;
// Largest number of frames one work unit of the shared-memory path handles.
constexpr uint32_t kMaxUnitFrames = 1024;

struct ChainParams {
  const uint8_t* flags;            // per frame of the block: gates holding data
  GateParams g;
  const float* baselines;          // [npol][2]: G0, G1 baselines used for this block
  unsigned long long* pol_stats;   // [npol][kPolStats]
  unsigned long long* sat;         // [n_out][2] saturation counts (G0, G1)
  uint8_t* out;                    // output accumulation buffer, host layout
  float* partial;                  // [n_out][slices][VALS][C] (slices > 1)
  const float2* tw;                // Stockham tables of the FFT length (small path)
  uint64_t out_rec;                // bytes per output record
  uint32_t n_out;
  uint32_t nacc;                   // frames per output spectrum per block
  uint32_t slices;                 // work units per output spectrum
  uint32_t frames_per_unit;
  uint32_t* dev_err;               // set non-zero when a bounded device wait gives up
  volatile uint32_t* err_host;     // page-locked mirror of *dev_err written by the finalisation (or null)
  uint32_t store;                  // 1: one block per output, so each launch writes every spectrum value of
                                   // its records (stores, no read-add); only the counters start from zero
  // finalisation by the chain's last CTA instead of a finalize launch (warp chain; ticket null: off)
  uint32_t* ticket;                // CTAs done with the block, modulo the grid size (zero between launches)
  float* fin_baselines;            // the block finalisation's baselines_out
  int32_t fin_convention, fin_ungated;
};

// Large-N (four-step) parameters.
struct FourStepParams {
  ChainParams c;
  float2* scratch;                 // [frames][SEQ][N1][N2] complex after pass A
  const float2* tw1;               // Stockham tables of N1
  const float2* tw2;               // Stockham tables of N2
  const float2* twA;               // W_N^(m_hi * 1024) , m_hi < N/1024
  const float2* twB;               // W_N^(m_lo), m_lo < 1024
  uint32_t N1, N2;                 // N = N1 * N2; input sample n = N2*n1 + n2
  uint32_t k0, nk;                 // output spectra of this launch
  uint32_t maxjobs;                // job slots per output spectrum
  uint32_t* jobs;                  // [n_out][maxjobs] job list per output spectrum
  uint32_t* njobs;                 // [n_out]
  uint32_t* dc;                    // [n_out][2] frames without data per gate
  unsigned long long* dcsum;       // [n_out][maxjobs][6] exact DC sums of each job (see exact_dc)
  float* bsum;                     // pass B row-pair sums of the launch: [nk][N1/2][VALS][N2 + 1]
  // tensor-core form (form != 0): DFT-32 operand parts and W1024 twiddles
  uint32_t form;                   // GSPEC_FORM_*
  const uint4* tc_img;             // [B1 | B2 | B3 | W1024] in shared-memory layout
};

// Host-side launchers (gspec_kernels.cu).
// Shared-memory path shapes run by the warp chain (one FFT per warp): single-pol 1024-point frames.
constexpr bool uses_warp_chain(int N, bool dual) { return N == 1024 && !dual; }
cudaError_t launch_small_chain(int N, int nbits, bool dual, const ChainParams& p, cudaStream_t s);
cudaError_t launch_reduce_finalize(int N, bool dual, const ChainParams& p, int npol, int convention, int ungated,
                                   float* baselines_out, cudaStream_t s);
cudaError_t launch_finalize(const ChainParams& p, int npol, int C, int dual, int convention, int ungated,
                            float* baselines_out, cudaStream_t s);
// Twiddle tables of the shared-memory path: the Stockham tables of N, and
// at N = 1024 the warp chain's stage table after them (small_tw_size entries).
cudaError_t launch_twiddles(int N, float2* tw, cudaStream_t s);
__host__ __device__ constexpr int small_tw_size(int N) { return tw_size(N) + (N == 1024 ? 1024 : 0); }
cudaError_t launch_fourstep_twiddles(int N, float2* twA, float2* twB, cudaStream_t s);
cudaError_t launch_gate_debug(int nbits, const GateParams& g, const float* baselines, int npol, uint32_t nsamps,
                              float* out, cudaStream_t s);
cudaError_t launch_unpack(int nbits, const uint8_t* raw, uint64_t nsamples, float* out, cudaStream_t s);
// One store of *src into device-accessible host memory dst.
// bytes (a multiple of 8) from device memory to device-accessible host memory by SM stores.
cudaError_t launch_copy_words(void* dst, const void* src, uint64_t bytes, int sm_count, cudaStream_t s);
cudaError_t launch_fourstep(int N, int nbits, bool dual, const FourStepParams& p, int pass, cudaStream_t s);
// masks of every item; per-frame gate flags when flags != nullptr
cudaError_t launch_prepass(const GateParams& g, uint32_t nitems, uint8_t* masks, uint32_t N, uint32_t nframes,
                           uint8_t* flags, cudaStream_t s);

int small_fft_threads(int N, bool dual);
size_t small_fft_smem(int N, bool dual);
bool small_fft_supported(int N);
bool fourstep_supported(int N);
int fourstep_n1(int N);
int fourstep_n2(int N);

}  // namespace gspec
