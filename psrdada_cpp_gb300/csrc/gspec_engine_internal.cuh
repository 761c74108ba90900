// Internal definitions shared by the host engine (gspec_engine.cu) and the
// allocation-free entry point (gspec_noalloc.cu).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "../../include/gspec.h"
#include "gspec_kernels.cuh"


using gspec::kMaxUnitFrames;
constexpr int kKernelKinds = 8;

struct gspec_handle {
  gspec_config cfg{};
  // layout (edd/src/DadaBufferLayout.cpp:17-39)
  uint64_t n_heaps = 0, gap = 0, data_bytes = 0, sc_off = 0, sc_bytes = 0;
  // derived (edd/detail/GatedSpectrometer.cu:99-153)
  uint64_t nsamps = 0, items_per_pol = 0, n_blocks = 1, batch = 0, nacc = 0, n_out = 0, C = 0;
  uint64_t rec = 0, out_bytes = 0, ext_bytes = 0, hand_bytes = 0;
  int npol = 1;
  bool dual = false;
  bool ungated = false;            // GSPEC_FLAG_UNGATED: the FftSpectrometer form
  int path = 0;
  uint32_t N1 = 0, N2 = 0;
  uint32_t slices = 1, frames_per_unit = 1;
  uint32_t kchunk = 1;
  int sm_count = 152;
  std::string err;

  uint8_t* d_in[2] = {nullptr, nullptr};
  uint8_t* d_out[2] = {nullptr, nullptr};
  unsigned long long* d_sat[2] = {nullptr, nullptr};
  unsigned long long* d_sat_dev = nullptr;
  char* h_out[2] = {nullptr, nullptr};
  char* h_out_dev[2] = {nullptr, nullptr};   // their device addresses (SM-store output copies)
  float* d_baselines = nullptr;
  unsigned long long* d_pol_stats = nullptr;
  float2* d_tw = nullptr;
  float2* d_tw1 = nullptr;
  float2* d_tw2 = nullptr;
  float2* d_twA = nullptr;
  float2* d_twB = nullptr;
  float* d_partial = nullptr;
  float2* d_scratch = nullptr;
  uint8_t* d_masks = nullptr;      // per side-channel item index: gates
  uint8_t* d_flags = nullptr;      // per frame: gates holding data
  uint32_t* d_jobs = nullptr;      // four-step job lists [kchunk][maxjobs]
  uint32_t* d_njobs = nullptr;
  uint32_t* d_dc = nullptr;
  unsigned long long* d_dcsum = nullptr;   // four-step: exact DC sums per job
  uint16_t* d_tc_parts = nullptr;  // tensor-core form: DFT-32 operand parts
  float2* d_tc_w = nullptr;        // W1024 twiddles
  uint8_t* d_tc_img = nullptr;     // [B1 | B2 | B3 | W1024] in shared-memory layout
  float* d_bsum = nullptr;         // pass-B row-pair sums of one chunk
  uint32_t maxjobs = 0;
  int32_t heap_shift = -1;
  uint32_t* d_err = nullptr;       // set by kernels whose bounded waits gave up
  uint32_t* d_ticket = nullptr;    // warp chain with whole spectra per CTA: CTAs done (its last one finalises)
  uint32_t* h_err = nullptr;       // pinned copy, refreshed after every block
  uint32_t* h_err_dev = nullptr;   // its device address (written by the block's finalisation)
  cudaStream_t h2d = nullptr, proc = nullptr, d2h = nullptr;
  cudaEvent_t ev_h2d[2] = {}, ev_in_free[2] = {}, ev_out_ready[2] = {};
  int ia = 1, oa = 0, ha = 0, handed = -1;
  bool host_written[2] = {false, false};
  // launch accounting and optional per-kernel event timing
  uint64_t launches = 0;
  uint64_t kind_launches[kKernelKinds] = {};
  int profiling = 0;
  struct Pending {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<Pending> pending;
  double kind_ms[kKernelKinds] = {};
  uint64_t kind_timed[kKernelKinds] = {};
  uint64_t call_count = 0;
  uint64_t device_bytes = 0;
};


namespace gspec_engine {
// Validates h->cfg and fills the derived sizes (no CUDA call).
bool configure_handle(gspec_handle* h);
// Slices per output spectrum of the shared-memory path (needs h->sm_count).
bool plan_units(gspec_handle* h);
// SM count, work units / scratch chunk (after configure_handle).
bool plan_handle(gspec_handle* h);
// The chain's last CTA finalises the block (warp chain, whole spectra per CTA).
bool fused_finalize(const gspec_handle* h);
// One block per output then writes every word of its records (no clearing).
bool path0_stores_records(const gspec_handle* h);
// Device bytes gspec_create allocates for a planned handle.
uint64_t footprint(const gspec_handle* h);
uint64_t bsum_bytes(const gspec_handle* h);
void fill_info(const gspec_handle* h, gspec_info* info);
// Clears an output buffer of h's layout for the first block of an output
// block (only the counters when each block holds whole outputs).
cudaError_t clear_output(const gspec_handle* h, uint8_t* d_out, cudaStream_t s);
// Enqueues the whole chain for one block on stream s using h's buffers.
cudaError_t run_chain(gspec_handle* h, const uint8_t* d_block, uint8_t* d_out, unsigned long long* d_sat,
                      cudaStream_t s);
}  // namespace gspec_engine
