// Host engine of the gated spectrometer and the C ABI of include/gspec.h.
//
// Mirrors GatedSpectrometer::operator() (edd/detail/GatedSpectrometer.cu:299-365):
// block n is copied to the device at call n, processed at call n+1,
// copied to the host at the next output swap and handed out one swap later,
// so the sequence of handler calls and their contents is the reference's.
// Differences: one H2D of the whole block per call (the dual-pol heap and
// item de-interleave of edd/src/GatedSpectrometer.cu:261-306 happens in the
// kernels' address arithmetic), one D2H per output block instead of 4*nOut
// or 16*nOut small copies (:346-384, :430-527), the input block is consumed
// before the call returns, and processing does not stall the host.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/gspec.h"
#include "gspec_kernels.cuh"

#include "gspec_engine_internal.cuh"
#include "gspec_tc_kernels.cuh"

using namespace gspec;

namespace {

int set_err(gspec_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  return code;
}

bool cuda_ok(gspec_handle* h, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  if (h) h->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

template <typename T>
bool dalloc(gspec_handle* h, T** p, size_t bytes, const char* what) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), bytes);
  if (e != cudaSuccess) {
    h->err = std::string("cudaMalloc ") + what + ": " + cudaGetErrorString(e);
    return false;
  }
  h->device_bytes += bytes;
  return true;
}

int group_bytes(int nbits) { return nbits == 8 ? 8 : (nbits == 10 ? 40 : 24); }
int group_samples(int nbits) { return nbits == 8 ? 8 : (nbits == 10 ? 32 : 16); }

// Validates the configuration and fills the derived sizes.
bool configure(gspec_handle* h) {
  auto fail = [&](const std::string& m) {
    h->err = m;
    return false;
  };
  // the ungated FFT spectrometer: the whole block is one "heap" of samples
  // with one virtual side-channel item that puts every sample into gate 0
  h->ungated = (h->cfg.flags & GSPEC_FLAG_UNGATED) != 0;
  if (h->ungated) {
    if (h->cfg.n_side_channels != 0) return fail("the ungated spectrometer's blocks hold samples only (n_side_channels 0)");
    if (h->cfg.input_type != GSPEC_SINGLE_POL || h->cfg.output_type != GSPEC_POWER)
      return fail("the ungated spectrometer takes single-pol samples and gives power spectra");
    if (h->cfg.convention != GSPEC_INTENDED) return fail("the ungated spectrometer has no gate convention");
    h->cfg.heap_size = h->cfg.buffer_size;
    h->cfg.selected_side_channel = 0;
    h->cfg.selected_bit = 0;
  }
  const gspec_config& c = h->cfg;
  if (c.nbits != 8 && c.nbits != 10 && c.nbits != 12) return fail("nbits must be 8, 10 or 12");
  if (c.input_type > 1 || c.output_type > 1) return fail("unknown input or output type");
  if (c.input_type == GSPEC_DUAL_POL && c.output_type == GSPEC_POWER)
    return fail("dual-pol power output is not implemented (as in the reference)");
  if (c.input_type == GSPEC_SINGLE_POL && c.output_type == GSPEC_FULL_STOKES)
    return fail("full-Stokes output needs dual-pol input");
  if (c.convention > 1) return fail("unknown gate convention");
  if (c.naccumulate == 0) return fail("naccumulate must be > 0");
  if (c.selected_bit >= 64) return fail("selected_bit must be < 64");
  if (c.n_side_channels == 0 && !h->ungated) return fail("at least one side-channel item per heap is required");
  if (c.selected_side_channel >= c.n_side_channels && !h->ungated) return fail("selected_side_channel out of range");
  if (c.heap_size == 0) return fail("heap_size must be > 0");
  const uint64_t N = c.fft_length;
  if (N == 0 || (N & (N - 1))) return fail("fft_length must be a power of two");
  if (small_fft_supported(static_cast<int>(N))) {
    h->path = 0;
  } else if (fourstep_supported(static_cast<int>(N))) {
    h->path = 1;
    h->N1 = fourstep_n1(static_cast<int>(N));
    h->N2 = fourstep_n2(static_cast<int>(N));
    if (c.form != GSPEC_FORM_FP32) {
      // the tensor-core passes are 1024 points long
      if (N >= (1u << 17)) {
        h->N1 = 1024;
        h->N2 = static_cast<uint32_t>(N / 1024);
      } else if (N == (1u << 16)) {
        h->N1 = 64;
        h->N2 = 1024;
      }
    }
    if (c.tune_n1) {
      const uint64_t n1 = c.tune_n1;
      if ((n1 & (n1 - 1)) || n1 < 64 || n1 > 1024 || N % n1 || N / n1 < 128 || N / n1 > 1024)
        return fail("tune_n1 must be a power of two in [64, 1024] with fft_length/tune_n1 in [128, 1024]");
      h->N1 = static_cast<uint32_t>(n1);
      h->N2 = static_cast<uint32_t>(N / n1);
    }
  } else {
    return fail("fft_length must be in [32, 2^20]");
  }
  if (c.form > GSPEC_FORM_FP16) return fail("unknown arithmetic form");
  if (c.form != GSPEC_FORM_FP32 && (h->path != 1 || (h->N1 != 1024 && h->N2 != 1024)))
    return fail("the tensor-core forms need fft_length 2^16..2^20 with a 1024-point four-step pass");
  h->dual = c.input_type == GSPEC_DUAL_POL;
  h->npol = h->dual ? 2 : 1;
  const uint64_t scs = c.n_side_channels * 8;
  h->n_heaps = c.buffer_size / (c.heap_size + scs);
  if (h->n_heaps == 0) return fail("buffer holds no heap");
  h->gap = c.buffer_size - h->n_heaps * (c.heap_size + scs);
  h->data_bytes = h->n_heaps * c.heap_size;
  h->sc_off = h->data_bytes + h->gap;
  h->sc_bytes = scs * h->n_heaps;
  if (h->dual && (h->n_heaps % 2)) return fail("dual-pol blocks need an even number of heaps");
  const uint64_t pol_bytes = h->dual ? h->data_bytes / 2 : h->data_bytes;
  if ((pol_bytes * 8) % c.nbits) return fail("pol data is not a whole number of samples");
  h->nsamps = pol_bytes * 8 / c.nbits;
  if (h->nsamps >= (1ull << 32)) return fail("more than 2^32 samples per pol");
  if (pol_bytes >= (1ull << 32)) return fail("more than 4 GiB of samples per pol in one block");
  h->items_per_pol = h->dual ? h->n_heaps * c.n_side_channels / 2 : h->n_heaps * c.n_side_channels;
  if (h->ungated) h->items_per_pol = 1;
  const int gb = group_bytes(c.nbits);
  if (h->dual && (c.heap_size % gb)) {
    return fail("dual-pol heap size must be a multiple of " + std::to_string(gb) + " bytes");
  }
  if (c.heap_size < static_cast<uint64_t>(gb)) return fail("heap smaller than one unpack group");
  // samples per heap as a shift when it is an integer power of two
  h->heap_shift = -1;
  if ((8 * c.heap_size) % c.nbits == 0) {
    const uint64_t sph = 8 * c.heap_size / c.nbits;
    if ((sph & (sph - 1)) == 0) {
      int sh = 0;
      while ((1ull << sh) < sph) ++sh;
      h->heap_shift = sh;
    }
  }
  // edd/detail/GatedSpectrometer.cu:114-130
  const uint64_t per_out = N * c.naccumulate;
  if (per_out <= h->nsamps) {
    if (h->nsamps % per_out) return fail("samples per pol not a multiple of fft_length*naccumulate");
    h->n_blocks = 1;
  } else {
    if (per_out % h->nsamps) return fail("fft_length*naccumulate not a multiple of samples per pol");
    h->n_blocks = per_out / h->nsamps;
    if (c.naccumulate % h->n_blocks || h->nsamps % N) return fail("block does not hold whole spectra");
  }
  h->batch = h->nsamps / N;
  h->nacc = c.naccumulate / h->n_blocks;
  h->n_out = h->batch / h->nacc;
  h->C = N / 2 + 1;
  h->rec = (h->dual ? 8 : 2) * (h->C * 4 + 8);
  h->out_bytes = h->rec * h->n_out;
  // handed to the handler: the records, or the gate-0 spectra alone
  h->hand_bytes = h->ungated ? h->n_out * h->C * 4 : h->out_bytes;
  h->ext_bytes = h->n_out * 16;
  if (c.convention == GSPEC_REFERENCE) {
    const uint64_t L = h->nsamps / h->n_out;
    const uint64_t step = h->items_per_pol / h->n_out;
    if (step * 4096 != L) return fail("reference gating: chunk offset step*4096 does not tile the block");
    const uint64_t last = (h->n_out - 1) * step + ((L - 1) / c.heap_size) * c.n_side_channels + c.selected_side_channel;
    if (last >= h->items_per_pol) return fail("reference gating: side-channel index runs past the item array");
  } else {
    const uint64_t last = ((h->nsamps - 1) * c.nbits / (8 * c.heap_size)) * c.n_side_channels + c.selected_side_channel;
    if (last >= h->items_per_pol) return fail("side-channel index runs past the item array");
  }
  return true;
}

GateParams gate_params(const gspec_handle* h, const uint8_t* block) {
  GateParams g{};
  g.block = block;
  g.sc_offset = h->sc_off;
  g.heap_size = static_cast<uint32_t>(h->cfg.heap_size);
  g.heap_magic = g.heap_size > 1 ? UINT64_MAX / g.heap_size + 1 : 0;   // ceil(2^64 / heap_size)
  g.nsc = static_cast<uint32_t>(h->cfg.n_side_channels);
  g.sel = static_cast<uint32_t>(h->cfg.selected_side_channel);
  g.bitpos = static_cast<uint32_t>(h->cfg.selected_bit);
  g.dual = h->dual ? 1u : 0u;
  g.convention = h->cfg.convention;
  g.chunk = static_cast<uint32_t>(h->nsamps / h->n_out);
  g.step = static_cast<uint32_t>(h->items_per_pol / h->n_out);
  g.nbits = h->cfg.nbits;
  g.heap_shift = h->heap_shift;
  g.masks = h->d_masks;
  g.win16 = (h->cfg.buffer_size % 16 == 0 && reinterpret_cast<uintptr_t>(block) % 16 == 0) ? 1u : 0u;
  return g;
}

const char* const kKernelNames[kKernelKinds] = {"small_chain", "reduce_finalize", "fourstep_a",      "fourstep_b",
                                                "finalize",    "gate_prepass",    "fourstep_scatter", "fourstep_plan"};

// Launches one kernel of the chain; with profiling on, brackets it with
// events on its own stream so per-kernel device time can be read back.
template <typename F>
cudaError_t timed(gspec_handle* h, int kind, cudaStream_t s, F&& launch) {
  ++h->launches;
  ++h->kind_launches[kind];
  if (!h->profiling) return launch();
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, s);
  cudaError_t e = launch();
  cudaEventRecord(b, s);
  h->pending.push_back({kind, a, b});
  return e;
}

// Error status of the kernels that completed so far.
int device_error(gspec_handle* h) {
  if (h->h_err && *h->h_err) {
    h->err = "a bounded device wait gave up (code " + std::to_string(*h->h_err) + ")";
    return GSPEC_ERR_CUDA;
  }
  return GSPEC_OK;
}

cudaError_t launch_chain(gspec_handle* h, const uint8_t* d_block, uint8_t* d_out, unsigned long long* d_sat,
                         cudaStream_t s) {
  ChainParams p{};
  p.g = gate_params(h, d_block);
  p.baselines = h->d_baselines;
  p.pol_stats = h->d_pol_stats;
  p.sat = d_sat;
  p.out = d_out;
  p.partial = h->d_partial;
  p.tw = h->d_tw;
  p.out_rec = h->rec;
  p.n_out = static_cast<uint32_t>(h->n_out);
  p.nacc = static_cast<uint32_t>(h->nacc);
  p.slices = h->slices;
  p.frames_per_unit = h->frames_per_unit;
  p.flags = h->d_flags;
  p.dev_err = h->d_err;
  p.err_host = h->d_err ? h->h_err_dev : nullptr;   // refreshed by the block's finalisation
  // each block holds whole outputs: every spectrum value is written once per block
  p.store = h->n_blocks == 1 ? 1u : 0u;
  const int N = static_cast<int>(h->cfg.fft_length);
  cudaError_t e;
  // gate masks per item and the gates each frame holds data in
  if (h->ungated) {
    // one item, in gate 0; every frame holds gate-0 data only
    e = cudaMemsetAsync(h->d_masks, 1, 1, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->d_flags, 1, h->batch, s);
  } else {
    e = timed(h, 5, s, [&] {
      return launch_prepass(p.g, static_cast<uint32_t>(h->items_per_pol), h->d_masks, static_cast<uint32_t>(N),
                            static_cast<uint32_t>(h->batch), h->d_flags, s);
    });
  }
  if (e != cudaSuccess) return e;
  if (h->path == 0) {
    if (h->d_ticket) {
      // the chain's last CTA finalises the block (no finalize launch)
      p.ticket = h->d_ticket;
      p.fin_baselines = h->d_baselines;
      p.fin_convention = static_cast<int32_t>(h->cfg.convention);
      p.fin_ungated = h->ungated ? 1 : 0;
      return timed(h, 0, s, [&] { return launch_small_chain(N, h->cfg.nbits, h->dual, p, s); });
    }
    e = timed(h, 0, s, [&] { return launch_small_chain(N, h->cfg.nbits, h->dual, p, s); });
    if (e != cudaSuccess) return e;
    if (h->slices > 1) {
      // partial spectra of the slices, then the baselines of the next block
      return timed(h, 1, s, [&] {
        return launch_reduce_finalize(N, h->dual, p, h->npol, static_cast<int>(h->cfg.convention),
                                      h->ungated ? 1 : 0, h->d_baselines, s);
      });
    }
  } else {
    FourStepParams f{};
    f.c = p;
    f.scratch = h->d_scratch;
    f.bsum = h->d_bsum;
    f.tw1 = h->d_tw1;
    f.tw2 = h->d_tw2;
    f.twA = h->d_twA;
    f.twB = h->d_twB;
    f.N1 = h->N1;
    f.N2 = h->N2;
    f.maxjobs = h->maxjobs;
    f.form = h->cfg.form;
    f.tc_img = reinterpret_cast<const uint4*>(h->d_tc_img);
    f.jobs = h->d_jobs;
    f.njobs = h->d_njobs;
    f.dc = h->d_dc;
    f.dcsum = h->d_dcsum;
    // job lists of every output spectrum of the block
    f.k0 = 0;
    f.nk = static_cast<uint32_t>(h->n_out);
    // the exact DC sums of every job are accumulated by pass A
    e = cudaMemsetAsync(h->d_dcsum, 0, 6ull * h->n_out * h->maxjobs * sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    e = timed(h, 7, s, [&] { return launch_fourstep(N, h->cfg.nbits, h->dual, f, -1, s); });
    if (e != cudaSuccess) return e;
    for (uint64_t k0 = 0; k0 < h->n_out; k0 += h->kchunk) {
      const uint64_t nk = std::min<uint64_t>(h->kchunk, h->n_out - k0);
      f.k0 = static_cast<uint32_t>(k0);
      f.nk = static_cast<uint32_t>(nk);
      e = timed(h, 2, s, [&] { return launch_fourstep(N, h->cfg.nbits, h->dual, f, 0, s); });
      if (e != cudaSuccess) return e;
      e = timed(h, 3, s, [&] { return launch_fourstep(N, h->cfg.nbits, h->dual, f, 1, s); });
      if (e != cudaSuccess) return e;
      e = timed(h, 6, s, [&] { return launch_fourstep(N, h->cfg.nbits, h->dual, f, 2, s); });
      if (e != cudaSuccess) return e;
    }
  }
  return timed(h, 4, s, [&] {
    return launch_finalize(p, h->npol, static_cast<int>(h->C), h->dual ? 1 : 0, static_cast<int>(h->cfg.convention),
                           h->ungated ? 1 : 0, h->d_baselines, s);
  });
}

uint64_t env_u64(const char* name, uint64_t dflt) {
  const char* v = std::getenv(name);
  if (!v || !*v) return dflt;
  return std::strtoull(v, nullptr, 10);
}

void release(gspec_handle* h) {
  if (!h) return;
  for (auto& p : h->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  h->pending.clear();
  for (int i = 0; i < 2; ++i) {
    if (h->d_in[i]) cudaFree(h->d_in[i]);
    if (h->d_out[i]) cudaFree(h->d_out[i]);
    if (h->d_sat[i]) cudaFree(h->d_sat[i]);
    if (h->h_out[i]) cudaFreeHost(h->h_out[i]);
    if (h->ev_h2d[i]) cudaEventDestroy(h->ev_h2d[i]);
    if (h->ev_in_free[i]) cudaEventDestroy(h->ev_in_free[i]);
    if (h->ev_out_ready[i]) cudaEventDestroy(h->ev_out_ready[i]);
  }
  void* ptrs[] = {h->d_sat_dev, h->d_baselines, h->d_pol_stats, h->d_tw,   h->d_tw1,   h->d_tw2,  h->d_twA,
                  h->d_twB,     h->d_partial,   h->d_scratch,   h->d_masks, h->d_flags, h->d_jobs, h->d_njobs,
                  h->d_dc,      h->d_err,       h->d_tc_parts,  h->d_tc_w,  h->d_tc_img, h->d_bsum,
                  h->d_dcsum,   h->d_ticket};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (h->h_err) cudaFreeHost(h->h_err);
  if (h->h2d) cudaStreamDestroy(h->h2d);
  if (h->proc) cudaStreamDestroy(h->proc);
  if (h->d2h) cudaStreamDestroy(h->d2h);
}

// Output blocks up to this size go to the pinned host buffer by SM stores.
#ifndef GSPEC_STORE_OUTPUT_MAX_MB
#define GSPEC_STORE_OUTPUT_MAX_MB 64
#endif
constexpr uint64_t kStoreOutputMax = static_cast<uint64_t>(GSPEC_STORE_OUTPUT_MAX_MB) << 20;

int do_process(gspec_handle* h, const void* block, size_t used, gspec_output* out, bool on_device) {
  if (!h || !out) return GSPEC_ERR_ARG;
  out->ready = 0;
  out->data = nullptr;
  out->size = 0;
  if (cudaSetDevice(h->cfg.device) != cudaSuccess) return set_err(h, GSPEC_ERR_CUDA, "cudaSetDevice failed");
  ++h->call_count;
  if (used != h->cfg.buffer_size) {
    cudaStreamSynchronize(h->h2d);
    cudaStreamSynchronize(h->proc);
    cudaStreamSynchronize(h->d2h);
    return set_err(h, GSPEC_STOP,
                   "Unexpected Buffer Size - Got " + std::to_string(used) + " byte, expected " +
                       std::to_string(h->cfg.buffer_size) + " byte");
  }
  if (!block) return set_err(h, GSPEC_ERR_ARG, "null block");
  if (!h->h_out[0]) return set_err(h, GSPEC_ERR_STATE, "handle was created with GSPEC_FLAG_NO_HOST_BUFFERS");
  // input double buffer: buffer a receives block n (edd/detail/GatedSpectrometer.cu:314-316)
  h->ia ^= 1;
  const int ia = h->ia, ib = ia ^ 1;
  if (!cuda_ok(h, cudaStreamWaitEvent(h->h2d, h->ev_in_free[ia], 0), "wait input") ||
      !cuda_ok(h, cudaMemcpyAsync(h->d_in[ia], block, h->cfg.buffer_size,
                                  on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, h->h2d),
               "H2D block") ||
      !cuda_ok(h, cudaEventRecord(h->ev_h2d[ia], h->h2d), "record h2d"))
    return GSPEC_ERR_CUDA;
  if (h->call_count == 1) {
    return cuda_ok(h, cudaStreamSynchronize(h->h2d), "H2D") ? GSPEC_OK : GSPEC_ERR_CUDA;
  }
  const bool new_block = ((h->call_count - 1) % h->n_blocks) == 0;
  if (new_block) {
    if (!cuda_ok(h, cudaStreamSynchronize(h->d2h), "D2H")) return GSPEC_ERR_CUDA;
    h->oa ^= 1;
    h->ha ^= 1;
    if (!cuda_ok(h, gspec_engine::clear_output(h, h->d_out[h->oa], h->proc), "clear output") ||
        !cuda_ok(h, cudaMemsetAsync(h->d_sat[h->oa], 0, h->ext_bytes, h->proc), "zero saturation"))
      return GSPEC_ERR_CUDA;
  }
  if (!cuda_ok(h, cudaStreamWaitEvent(h->proc, h->ev_h2d[ib], 0), "wait h2d") ||
      !cuda_ok(h, launch_chain(h, h->d_in[ib], h->d_out[h->oa], h->d_sat[h->oa], h->proc), "chain kernels") ||
      !cuda_ok(h, cudaEventRecord(h->ev_in_free[ib], h->proc), "record input free") ||
      !cuda_ok(h, cudaEventRecord(h->ev_out_ready[h->oa], h->proc), "record output"))
    return GSPEC_ERR_CUDA;
  if (!(h->call_count == 2 || !new_block)) {
    const int ob = h->oa ^ 1;
    if (!cuda_ok(h, cudaStreamWaitEvent(h->d2h, h->ev_out_ready[ob], 0), "wait output")) return GSPEC_ERR_CUDA;
    if (h->ungated) {
      // the gate-0 spectrum of every record, packed (FftSpectrometer's output)
      if (!cuda_ok(h, cudaMemcpy2DAsync(h->h_out[h->ha], h->C * 4, h->d_out[ob], h->rec, h->C * 4, h->n_out,
                                        cudaMemcpyDeviceToHost, h->d2h),
                   "D2H spectra") ||
          !cuda_ok(h, cudaMemcpyAsync(h->h_out[h->ha] + h->hand_bytes, h->d_sat[ob], h->ext_bytes,
                                      cudaMemcpyDeviceToHost, h->d2h),
                   "D2H saturation"))
        return GSPEC_ERR_CUDA;
    } else if (h->out_bytes + h->ext_bytes <= kStoreOutputMax) {
      // SM stores into the pinned buffer: the host link then keeps its full
      // host-to-device rate for the next block's copy (a copy engine in each
      // direction at once takes ~170 GB/s from each)
      if (!cuda_ok(h, gspec::launch_copy_words(h->h_out_dev[h->ha], h->d_out[ob], h->out_bytes, h->sm_count, h->d2h),
                   "output copy") ||
          !cuda_ok(h, gspec::launch_copy_words(h->h_out_dev[h->ha] + h->out_bytes, h->d_sat[ob], h->ext_bytes,
                                               h->sm_count, h->d2h),
                   "saturation copy"))
        return GSPEC_ERR_CUDA;
      h->launches += 2;
    } else if (!cuda_ok(h, cudaMemcpyAsync(h->h_out[h->ha], h->d_out[ob], h->out_bytes, cudaMemcpyDeviceToHost,
                                           h->d2h),
                        "D2H output") ||
               !cuda_ok(h, cudaMemcpyAsync(h->h_out[h->ha] + h->out_bytes, h->d_sat[ob], h->ext_bytes,
                                           cudaMemcpyDeviceToHost, h->d2h),
                        "D2H saturation")) {
      return GSPEC_ERR_CUDA;
    }
    h->host_written[h->ha] = true;
    // the reference also hands out the never-written buffer at the first
    // output swap when n_blocks >= 3; that call is skipped here
    if (h->call_count != 3 && h->host_written[h->ha ^ 1]) {
      h->handed = h->ha ^ 1;
      out->data = h->h_out[h->handed];
      out->size = h->hand_bytes + ((h->cfg.flags & GSPEC_FLAG_SATURATION_RECORD) ? h->ext_bytes : 0);
      out->ready = 1;
    }
  }
  // the ring buffer releases the block after the call returns
  if (!cuda_ok(h, cudaStreamSynchronize(h->h2d), "H2D")) return GSPEC_ERR_CUDA;
  if (device_error(h) != GSPEC_OK) return GSPEC_ERR_CUDA;
  if (!cuda_ok(h, cudaPeekAtLastError(), "CUDA")) return GSPEC_ERR_CUDA;
  return GSPEC_OK;
}

}  // namespace

namespace gspec_engine {

// What an output buffer needs cleared before the first block of an output
// block: with one block per output every spectrum value is stored by that
// block (ChainParams::store), so only each record's counters (added to by
// the block's atomics); otherwise the whole buffer.
cudaError_t clear_output(const gspec_handle* h, uint8_t* d_out, cudaStream_t s) {
  // the warp chain with whole spectra per CTA stores the counters as well
  if (h->n_blocks == 1 && path0_stores_records(h)) return cudaSuccess;
  if (h->n_blocks == 1) {
    const uint64_t spectra = (h->dual ? 8 : 2) * h->C * 4;
    return cudaMemset2DAsync(d_out + spectra, h->rec, 0, h->rec - spectra, h->n_out, s);
  }
  return cudaMemsetAsync(d_out, 0, h->out_bytes, s);
}

bool configure_handle(gspec_handle* h) { return configure(h); }

// Work units of the shared-memory path: output spectra are split into
// slices until there is about one unit per SM and no unit exceeds
// kMaxUnitFrames frames.  Whole spectra per unit need no partial sums: at
// fft 1024 / naccumulate 64 (256 spectra per block) one unit per spectrum
// runs the chain 8 % faster than four slices per spectrum.
bool plan_units(gspec_handle* h) {
  const uint64_t target = h->cfg.tune_units ? h->cfg.tune_units : env_u64("GSPEC_UNITS", h->sm_count);
  uint64_t s = env_u64("GSPEC_SLICES", 0);
  if (s == 0) {
    s = 1;
    while (h->n_out * s < target && h->nacc % (2 * s) == 0) s *= 2;
  }
  while (h->nacc / s > kMaxUnitFrames && h->nacc % (2 * s) == 0) s *= 2;
  if (h->nacc % s) {
    h->err = "GSPEC_SLICES must divide the frames per output spectrum";
    return false;
  }
  if (h->nacc / s > kMaxUnitFrames) {
    h->err = "more than 1024 frames per work unit";
    return false;
  }
  h->slices = static_cast<uint32_t>(s);
  h->frames_per_unit = static_cast<uint32_t>(h->nacc / s);
  return true;
}

cudaError_t run_chain(gspec_handle* h, const uint8_t* d_block, uint8_t* d_out, unsigned long long* d_sat,
                      cudaStream_t s) {
  return launch_chain(h, d_block, d_out, d_sat, s);
}

// Device-dependent planning after configure_handle: SM count, work units of
// the shared-memory path, job slots and scratch chunk of the four-step path.
bool plan_handle(gspec_handle* h) {
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, h->cfg.device) != cudaSuccess) {
    h->err = "cannot read the properties of device " + std::to_string(h->cfg.device);
    return false;
  }
  h->sm_count = prop.multiProcessorCount;
  if (h->path == 0) return plan_units(h);
  if (h->nacc > kMaxJobFrames) {
    h->err = "more than 16383 frames per output spectrum in one block";
    return false;
  }
  h->maxjobs = static_cast<uint32_t>(h->nacc * (h->dual ? 2 : 1));
  // scratch of the chunk of output spectra in flight
  const uint64_t mb = h->cfg.tune_scratch_mb ? h->cfg.tune_scratch_mb : env_u64("GSPEC_SCRATCH_MB", 512);
  const uint64_t per_out = static_cast<uint64_t>(h->maxjobs) * h->cfg.fft_length * sizeof(float2);
  uint64_t kc = (mb << 20) / per_out;
  if (kc < 1) kc = 1;
  if (kc > h->n_out) kc = h->n_out;
  h->kchunk = static_cast<uint32_t>(kc);
  return true;
}

// Pass-B row-pair sums of one chunk of output spectra (four-step path).
uint64_t bsum_bytes(const gspec_handle* h) {
  return static_cast<uint64_t>(h->kchunk) * (h->N1 / 2) * (h->dual ? 8 : 2) * (h->N2 + 1) * sizeof(float);
}

// The warp chain finalises the block in its last CTA when each CTA holds
// whole spectra (no partial sums to reduce first).
bool fused_finalize(const gspec_handle* h) {
  return h->path == 0 && h->slices == 1 && uses_warp_chain(static_cast<int>(h->cfg.fft_length), h->dual);
}

// With one block per output, the same chain stores every word of each
// record (spectra and counters), so the output needs no clearing.
bool path0_stores_records(const gspec_handle* h) { return fused_finalize(h); }

// Device bytes gspec_create allocates for a planned handle (the same list
// and the same 16-byte minimum as its dalloc calls).
uint64_t footprint(const gspec_handle* h) {
  auto sz = [](uint64_t b) { return b ? b : 16; };
  const uint64_t N = h->cfg.fft_length;
  const uint64_t vals = h->dual ? 8 : 2;
  uint64_t t = sz(h->items_per_pol) + sz(h->batch);
  t += 2 * (sz(h->cfg.buffer_size) + sz(h->out_bytes) + sz(h->ext_bytes));
  t += sz(h->ext_bytes) + sz(4 * sizeof(float)) + sz(2 * kPolStats * sizeof(unsigned long long)) + sz(sizeof(uint32_t));
  if (h->path == 0) {
    t += sz(small_tw_size(static_cast<int>(N)) * sizeof(float2));
    if (h->slices > 1) t += sz(h->n_out * h->slices * vals * h->C * sizeof(float));
    if (fused_finalize(h)) t += sz(sizeof(uint32_t));
  } else {
    t += sz(tw_size(static_cast<int>(h->N1)) * sizeof(float2)) + sz(tw_size(static_cast<int>(h->N2)) * sizeof(float2));
    t += 2 * sz(1024 * sizeof(float2));
    t += sz(static_cast<uint64_t>(h->kchunk) * h->maxjobs * N * sizeof(float2));
    t += sz(h->n_out * h->maxjobs * sizeof(uint32_t)) + sz(h->n_out * sizeof(uint32_t)) +
         sz(2ull * h->n_out * sizeof(uint32_t)) + sz(6ull * h->n_out * h->maxjobs * sizeof(unsigned long long));
    t += sz(bsum_bytes(h));
    if (h->cfg.form != GSPEC_FORM_FP32)
      t += sz(tc::kTableParts * 4096 * sizeof(uint16_t)) + sz(1024 * sizeof(float2)) + sz(tc::kImageBytesHost);
  }
  return t;
}

void fill_info(const gspec_handle* h, gspec_info* info) {
  info->nchans = h->C;
  info->n_out = h->n_out;
  info->n_blocks = h->n_blocks;
  info->nsamps_per_pol = h->nsamps;
  info->batch = h->batch;
  info->output_bytes = h->hand_bytes + ((h->cfg.flags & GSPEC_FLAG_SATURATION_RECORD) ? h->ext_bytes : 0);
  info->record_bytes = h->rec;
  info->device_bytes = h->device_bytes;
  info->fft_path = static_cast<uint64_t>(h->path);
  info->n1 = h->N1;
  info->n2 = h->N2;
  info->kernel_launches = h->launches;
}

}  // namespace gspec_engine

extern "C" {

gspec_handle* gspec_create(const gspec_config* cfg, char* err, size_t err_len) {
  auto report = [&](const std::string& m) {
    if (err && err_len) {
      std::snprintf(err, err_len, "%s", m.c_str());
    }
  };
  if (!cfg) {
    report("null config");
    return nullptr;
  }
  gspec_handle* h = new gspec_handle();
  h->cfg = *cfg;
  if (!configure(h)) {
    report(h->err);
    delete h;
    return nullptr;
  }
  auto bail = [&](const std::string& m) -> gspec_handle* {
    report(m.empty() ? h->err : m);
    release(h);
    delete h;
    return nullptr;
  };
  if (cudaSetDevice(cfg->device) != cudaSuccess) return bail("cudaSetDevice failed");
  if (!gspec_engine::plan_handle(h)) return bail("");
  int least = 0, greatest = 0;
  cudaDeviceGetStreamPriorityRange(&least, &greatest);
  int prio = cfg->stream_priority;
  if (prio > least) prio = least;
  if (prio < greatest) prio = greatest;
  if (!cuda_ok(h, cudaStreamCreateWithPriority(&h->h2d, cudaStreamNonBlocking, prio), "stream") ||
      !cuda_ok(h, cudaStreamCreateWithPriority(&h->proc, cudaStreamNonBlocking, prio), "stream") ||
      !cuda_ok(h, cudaStreamCreateWithPriority(&h->d2h, cudaStreamNonBlocking, prio), "stream"))
    return bail("");
  for (int i = 0; i < 2; ++i) {
    if (!cuda_ok(h, cudaEventCreateWithFlags(&h->ev_h2d[i], cudaEventDisableTiming), "event") ||
        !cuda_ok(h, cudaEventCreateWithFlags(&h->ev_in_free[i], cudaEventDisableTiming), "event") ||
        !cuda_ok(h, cudaEventCreateWithFlags(&h->ev_out_ready[i], cudaEventDisableTiming), "event"))
      return bail("");
  }
  const int N = static_cast<int>(cfg->fft_length);
  const uint64_t vals = h->dual ? 8 : 2;
  if (!dalloc(h, &h->d_masks, h->items_per_pol, "gate masks") || !dalloc(h, &h->d_flags, h->batch, "frame flags"))
    return bail("");
  for (int i = 0; i < 2; ++i) {
    if (!dalloc(h, &h->d_in[i], cfg->buffer_size, "input") || !dalloc(h, &h->d_out[i], h->out_bytes, "output") ||
        !dalloc(h, &h->d_sat[i], h->ext_bytes, "saturation"))
      return bail("");
    if (!(cfg->flags & GSPEC_FLAG_NO_HOST_BUFFERS)) {
      if (!cuda_ok(h, cudaMallocHost(reinterpret_cast<void**>(&h->h_out[i]), h->out_bytes + h->ext_bytes),
                   "pinned output"))
        return bail("");
      std::memset(h->h_out[i], 0, h->out_bytes + h->ext_bytes);
      if (!cuda_ok(h, cudaHostGetDevicePointer(reinterpret_cast<void**>(&h->h_out_dev[i]), h->h_out[i], 0),
                   "device address of the pinned output"))
        return bail("");
    }
    if (!cuda_ok(h, cudaMemset(h->d_out[i], 0, h->out_bytes), "memset") ||
        !cuda_ok(h, cudaMemset(h->d_sat[i], 0, h->ext_bytes), "memset"))
      return bail("");
  }
  if (!dalloc(h, &h->d_sat_dev, h->ext_bytes, "saturation") || !dalloc(h, &h->d_baselines, 4 * sizeof(float), "baselines") ||
      !dalloc(h, &h->d_pol_stats, 2 * kPolStats * sizeof(unsigned long long), "stats"))
    return bail("");
  cudaMemset(h->d_baselines, 0, 4 * sizeof(float));
  cudaMemset(h->d_pol_stats, 0, 2 * kPolStats * sizeof(unsigned long long));
  cudaMemset(h->d_sat_dev, 0, h->ext_bytes);
  if (!dalloc(h, &h->d_err, sizeof(uint32_t), "error word") ||
      !cuda_ok(h, cudaMallocHost(reinterpret_cast<void**>(&h->h_err), sizeof(uint32_t)), "pinned error word"))
    return bail("");
  *h->h_err = 0;
  if (!cuda_ok(h, cudaHostGetDevicePointer(reinterpret_cast<void**>(&h->h_err_dev), h->h_err, 0),
               "device address of the error word"))
    return bail("");
  cudaMemset(h->d_err, 0, sizeof(uint32_t));
  if (h->path == 0) {
    if (!dalloc(h, &h->d_tw, small_tw_size(N) * sizeof(float2), "twiddles")) return bail("");
    if (!cuda_ok(h, launch_twiddles(N, h->d_tw, h->proc), "twiddles")) return bail("");
    if (h->slices > 1 &&
        !dalloc(h, &h->d_partial, h->n_out * h->slices * vals * h->C * sizeof(float), "partials"))
      return bail("");
    if (gspec_engine::fused_finalize(h)) {
      if (!dalloc(h, &h->d_ticket, sizeof(uint32_t), "chain ticket")) return bail("");
      cudaMemset(h->d_ticket, 0, sizeof(uint32_t));
    }
  } else {
    if (!dalloc(h, &h->d_tw1, tw_size(h->N1) * sizeof(float2), "twiddles") ||
        !dalloc(h, &h->d_tw2, tw_size(h->N2) * sizeof(float2), "twiddles") ||
        !dalloc(h, &h->d_twA, 1024 * sizeof(float2), "twiddles") ||
        !dalloc(h, &h->d_twB, 1024 * sizeof(float2), "twiddles"))
      return bail("");
    if (!cuda_ok(h, launch_twiddles(h->N1, h->d_tw1, h->proc), "twiddles") ||
        !cuda_ok(h, launch_twiddles(h->N2, h->d_tw2, h->proc), "twiddles") ||
        !cuda_ok(h, launch_fourstep_twiddles(N, h->d_twA, h->d_twB, h->proc), "twiddles"))
      return bail("");
    const uint64_t slots = static_cast<uint64_t>(h->kchunk) * h->maxjobs;
    if (!dalloc(h, &h->d_scratch, slots * static_cast<uint64_t>(N) * sizeof(float2), "four-step scratch") ||
        !dalloc(h, &h->d_jobs, h->n_out * h->maxjobs * sizeof(uint32_t), "job lists") ||
        !dalloc(h, &h->d_njobs, h->n_out * sizeof(uint32_t), "job counts") ||
        !dalloc(h, &h->d_dc, 2ull * h->n_out * sizeof(uint32_t), "dc counts") ||
        !dalloc(h, &h->d_dcsum, 6ull * h->n_out * h->maxjobs * sizeof(unsigned long long), "dc sums") ||
        !dalloc(h, &h->d_bsum, gspec_engine::bsum_bytes(h), "pass-B sums"))
      return bail("");
    if (cfg->form != GSPEC_FORM_FP32) {
      if (!dalloc(h, &h->d_tc_parts, tc::kTableParts * 4096 * sizeof(uint16_t), "tensor-core operand") ||
          !dalloc(h, &h->d_tc_w, 1024 * sizeof(float2), "tensor-core twiddles") ||
          !dalloc(h, &h->d_tc_img, tc::kImageBytesHost, "tensor-core image"))
        return bail("");
      if (!cuda_ok(h, tc::launch_tables(h->d_tc_parts, h->d_tc_w, cfg->form == GSPEC_FORM_BF16, h->proc),
                   "tensor-core tables") ||
          !cuda_ok(h, tc::launch_image(h->d_tc_parts, h->d_tc_w, h->d_tc_img, h->proc), "tensor-core image"))
        return bail("");
    }
  }
  if (!cuda_ok(h, cudaStreamSynchronize(h->proc), "setup")) return bail("");
  return h;
}

void gspec_destroy(gspec_handle* h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  if (h->h2d) cudaStreamSynchronize(h->h2d);
  if (h->proc) cudaStreamSynchronize(h->proc);
  if (h->d2h) cudaStreamSynchronize(h->d2h);
  release(h);
  delete h;
}

int gspec_init(gspec_handle* h, char* header, size_t total_bytes) {
  if (!h || !header) return GSPEC_ERR_ARG;
  // FftSpectrometer::init only forwards the header (edd/detail/FftSpectrometer.cu:119-123)
  if (h->ungated) return GSPEC_OK;
  char text[512];
  const int n = std::snprintf(text, sizeof(text),
                              "\n# Gated spectrometer parameters: \n"
                              "fft_length               %llu\n"
                              "nchannels                %llu\n"
                              "naccumulate              %llu\n"
                              "selected_side_channel    %llu\n"
                              "selected_bit             %llu\n"
                              "output_bit_depth         %d\n"
                              "full_stokes_output       %s\n",
                              static_cast<unsigned long long>(h->cfg.fft_length),
                              static_cast<unsigned long long>(h->C),
                              static_cast<unsigned long long>(h->cfg.naccumulate),
                              static_cast<unsigned long long>(h->cfg.selected_side_channel),
                              static_cast<unsigned long long>(h->cfg.selected_bit), 32,
                              h->cfg.output_type == GSPEC_FULL_STOKES ? "yes" : "no");
  const size_t end = strnlen(header, total_bytes);
  if (end + static_cast<size_t>(n) < total_bytes) {
    std::memcpy(header + end, text, static_cast<size_t>(n) + 1);
    return GSPEC_OK;
  }
  h->err = "Header of size " + std::to_string(total_bytes) + " bytes already contains " + std::to_string(end) +
           " bytes. Cannot add gated spectrometer info of size " + std::to_string(n) + " bytes.";
  return GSPEC_STOP;
}

int gspec_process(gspec_handle* h, const char* block, size_t used_bytes, gspec_output* out) {
  return do_process(h, block, used_bytes, out, false);
}

int gspec_process_device(gspec_handle* h, const void* d_block, size_t used_bytes, gspec_output* out) {
  return do_process(h, d_block, used_bytes, out, true);
}

int gspec_clear_output_device(gspec_handle* h, void* d_out, void* cuda_stream) {
  if (!h || !d_out) return GSPEC_ERR_ARG;
  return cuda_ok(h, gspec_engine::clear_output(h, static_cast<uint8_t*>(d_out), static_cast<cudaStream_t>(cuda_stream)),
                 "clear output")
             ? GSPEC_OK
             : GSPEC_ERR_CUDA;
}

int gspec_run_block_device(gspec_handle* h, const void* d_block, void* d_out, void* cuda_stream) {
  if (!h || !d_block || !d_out) return GSPEC_ERR_ARG;
  // the kernels read the block in 8-byte words and add 8-byte counters to d_out
  if ((reinterpret_cast<uintptr_t>(d_block) | reinterpret_cast<uintptr_t>(d_out)) % 16)
    return set_err(h, GSPEC_ERR_ARG, "d_block and d_out must be 16-byte aligned");
  if (device_error(h) != GSPEC_OK) return GSPEC_ERR_CUDA;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  if (!cuda_ok(h, launch_chain(h, static_cast<const uint8_t*>(d_block), static_cast<uint8_t*>(d_out), h->d_sat_dev, s),
               "chain kernels"))
    return GSPEC_ERR_CUDA;
  return GSPEC_OK;
}

int gspec_get_info(const gspec_handle* h, gspec_info* info) {
  if (!h || !info) return GSPEC_ERR_ARG;
  gspec_engine::fill_info(h, info);
  return GSPEC_OK;
}

int gspec_query(const gspec_config* cfg, gspec_info* info, char* err, size_t err_len) {
  auto report = [&](const std::string& m) {
    if (err && err_len) std::snprintf(err, err_len, "%s", m.c_str());
  };
  if (!cfg || !info) {
    report("null argument");
    return GSPEC_ERR_ARG;
  }
  gspec_handle h;
  h.cfg = *cfg;
  if (!configure(&h)) {
    report(h.err);
    return GSPEC_ERR_ARG;
  }
  if (!gspec_engine::plan_handle(&h)) {
    report(h.err);
    return GSPEC_ERR_ARG;
  }
  h.device_bytes = gspec_engine::footprint(&h);
  gspec_engine::fill_info(&h, info);
  return GSPEC_OK;
}

const char* gspec_last_error(const gspec_handle* h) { return h ? h->err.c_str() : "null handle"; }

int gspec_set_profiling(gspec_handle* h, int enable) {
  if (!h) return GSPEC_ERR_ARG;
  h->profiling = enable ? 1 : 0;
  return GSPEC_OK;
}

int gspec_get_profile(gspec_handle* h, gspec_kernel_profile* out, int max_entries) {
  if (!h || !out) return GSPEC_ERR_ARG;
  if (!cuda_ok(h, cudaDeviceSynchronize(), "sync")) return GSPEC_ERR_CUDA;
  for (auto& p : h->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      h->kind_ms[p.kind] += ms;
      ++h->kind_timed[p.kind];
    }
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  h->pending.clear();
  int n = 0;
  for (int k = 0; k < kKernelKinds && n < max_entries; ++k) {
    std::snprintf(out[n].name, sizeof(out[n].name), "%s", kKernelNames[k]);
    out[n].launches = h->kind_launches[k];
    out[n].timed_launches = h->kind_timed[k];
    out[n].total_ms = h->kind_ms[k];
    ++n;
  }
  return n;
}

int gspec_reset_profile(gspec_handle* h) {
  if (!h) return GSPEC_ERR_ARG;
  gspec_kernel_profile tmp[kKernelKinds];
  gspec_get_profile(h, tmp, kKernelKinds);
  for (int k = 0; k < kKernelKinds; ++k) {
    h->kind_launches[k] = 0;
    h->kind_timed[k] = 0;
    h->kind_ms[k] = 0.0;
  }
  h->launches = 0;
  return GSPEC_OK;
}

int gspec_get_baselines(gspec_handle* h, float* out4) {
  if (!h || !out4) return GSPEC_ERR_ARG;
  if (!cuda_ok(h, cudaStreamSynchronize(h->proc), "sync") ||
      !cuda_ok(h, cudaMemcpy(out4, h->d_baselines, 4 * sizeof(float), cudaMemcpyDeviceToHost), "baselines"))
    return GSPEC_ERR_CUDA;
  return GSPEC_OK;
}

int gspec_set_baselines(gspec_handle* h, const float* in4) {
  if (!h || !in4) return GSPEC_ERR_ARG;
  if (!cuda_ok(h, cudaStreamSynchronize(h->proc), "sync") ||
      !cuda_ok(h, cudaMemcpy(h->d_baselines, in4, 4 * sizeof(float), cudaMemcpyHostToDevice), "baselines"))
    return GSPEC_ERR_CUDA;
  return GSPEC_OK;
}

int gspec_register_host(void* ptr, size_t bytes) {
  if (!ptr || !bytes) return GSPEC_ERR_ARG;
  return cudaHostRegister(ptr, bytes, cudaHostRegisterPortable | cudaHostRegisterMapped) == cudaSuccess
             ? GSPEC_OK
             : GSPEC_ERR_CUDA;
}

int gspec_unregister_host(void* ptr) {
  if (!ptr) return GSPEC_ERR_ARG;
  return cudaHostUnregister(ptr) == cudaSuccess ? GSPEC_OK : GSPEC_ERR_CUDA;
}

int gspec_get_saturation(gspec_handle* h, uint64_t* out) {
  if (!h || !out) return GSPEC_ERR_ARG;
  if (h->handed < 0) return set_err(h, GSPEC_ERR_STATE, "no output handed out yet");
  std::memcpy(out, h->h_out[h->handed] + h->hand_bytes, h->ext_bytes);
  return GSPEC_OK;
}

int gspec_unpack_device(const void* d_raw, uint32_t nbits, uint64_t nsamples, float* d_out, void* cuda_stream) {
  if (!d_raw || !d_out) return GSPEC_ERR_ARG;
  if (nbits != 8 && nbits != 10 && nbits != 12) return GSPEC_ERR_ARG;
  if (nsamples % group_samples(static_cast<int>(nbits))) return GSPEC_ERR_ARG;
  cudaError_t e = launch_unpack(static_cast<int>(nbits), static_cast<const uint8_t*>(d_raw), nsamples, d_out,
                                static_cast<cudaStream_t>(cuda_stream));
  return e == cudaSuccess ? GSPEC_OK : GSPEC_ERR_CUDA;
}

int gspec_gate_device(gspec_handle* h, const void* d_block, float* d_gated, void* cuda_stream) {
  if (!h || !d_block || !d_gated) return GSPEC_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  if (!cuda_ok(h, cudaStreamSynchronize(h->proc), "sync")) return GSPEC_ERR_CUDA;
  const GateParams g = gate_params(h, static_cast<const uint8_t*>(d_block));
  if (!cuda_ok(h, launch_prepass(g, static_cast<uint32_t>(h->items_per_pol), h->d_masks, 0, 0, nullptr, s),
               "mask kernel") ||
      !cuda_ok(h, launch_gate_debug(h->cfg.nbits, g, h->d_baselines, h->npol, static_cast<uint32_t>(h->nsamps),
                                    d_gated, s),
               "gate kernel"))
    return GSPEC_ERR_CUDA;
  return GSPEC_OK;
}

}  // extern "C"
