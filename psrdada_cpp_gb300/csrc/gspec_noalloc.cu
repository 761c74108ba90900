// Allocation-free entry point: one block through the gated-spectrometer
// chain with every working buffer carved from a fixed device array that the
// library owns.
//
// Some callers cannot allocate device memory on the hot path: a real-time
// DADA consumer whose device memory is all reserved up front by the ring
// buffer (dada_cuda_dbregister'ed blocks) and a pool it manages itself,
// processes running under a memory budget enforced by an outside allocator,
// or code that must never trigger the implicit device synchronisation and
// latency of cudaMalloc/cudaFree between blocks.  For them
// gspec_process_block_noalloc takes the device block, the baselines and the
// output buffer from the caller and uses gspec_noalloc_scratch below for the
// rest (gate masks, frame flags, twiddles, per-pol statistics, saturation
// counts and slice partials).  It calls no cudaMalloc, cudaFree or other
// allocating routine.
//
// The array is a file-scope __device__ object of GSPEC_NOALLOC_SCRATCH_BYTES
// (32 MiB): every GPU that loads the library holds it until the process
// exits.  Host code cannot use the array's name as a device address (in host
// code it names a host-side stand-in), so the first call on each device, with
// that device current, asks the runtime for the device address with
// cudaGetSymbolAddress and keeps it; that first call should therefore come
// before any stream capture.  Under CUDA's default lazy module loading the
// driver also reserves the array on the device at that first lookup, so a
// caller that reserves all remaining device memory for its own pool makes the
// first call at start-up, before reserving it.  The kept address belongs to
// the device's primary context; it is not refreshed after a cudaDeviceReset.
// All calls share the one array and it keeps the
// last call's contents: the per-pol statistics and saturation counts are
// cleared by every call, everything else is fully rewritten.  Calls whose
// work overlaps on the GPU (different streams, or different host threads)
// race on the array and must be serialised by the caller.
#include <cstdio>
#include <cstring>
#include <mutex>

#include "gspec_engine_internal.cuh"

namespace {

constexpr size_t kScratchBytes = GSPEC_NOALLOC_SCRATCH_BYTES;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char gspec_noalloc_scratch[kScratchBytes];

struct DeviceSlot {
  bool ready = false;
  unsigned char* base = nullptr;  // device address of gspec_noalloc_scratch
  int sm_count = 0;
};

std::mutex g_setup_mutex;
DeviceSlot g_slots[kMaxDevices];

int fail(char* err, size_t len, int code, const char* msg) {
  if (err && len) std::snprintf(err, len, "%s", msg);
  return code;
}

size_t align256(size_t n) { return (n + 255) & ~static_cast<size_t>(255); }

}  // namespace

extern "C" int gspec_process_block_noalloc(const gspec_config* cfg, const void* d_block, float* d_baselines,
                                           void* d_out, void* cuda_stream, char* err, size_t err_len) {
  if (!cfg || !d_block || !d_baselines || !d_out) return fail(err, err_len, GSPEC_ERR_ARG, "null argument");
  // the kernels read the block in 8-byte words and add 8-byte counters to d_out
  if ((reinterpret_cast<uintptr_t>(d_block) | reinterpret_cast<uintptr_t>(d_out)) % 16 ||
      reinterpret_cast<uintptr_t>(d_baselines) % 4)
    return fail(err, err_len, GSPEC_ERR_ARG, "d_block and d_out must be 16-byte aligned, d_baselines 4-byte");
  gspec_handle h;  // stack description only: no buffer of its own
  h.cfg = *cfg;
  if (!gspec_engine::configure_handle(&h)) return fail(err, err_len, GSPEC_ERR_ARG, h.err.c_str());
  if (h.path != 0)
    return fail(err, err_len, GSPEC_ERR_UNSUPPORTED,
                "gspec_process_block_noalloc handles fft_length <= 4096; longer transforms need the four-step "
                "scratch of a gspec_create handle");
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
    return fail(err, err_len, GSPEC_ERR_CUDA, "no current CUDA device");
  if (dev != cfg->device)
    return fail(err, err_len, GSPEC_ERR_ARG, "gspec_config.device must be the current CUDA device");

  // once per device, with that device current: the array's device address
  DeviceSlot slot;
  {
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    DeviceSlot& s = g_slots[dev];
    if (!s.ready) {
      void* p = nullptr;
      cudaError_t e = cudaGetSymbolAddress(&p, gspec_noalloc_scratch);
      if (e != cudaSuccess || !p) return fail(err, err_len, GSPEC_ERR_CUDA, "cudaGetSymbolAddress failed");
      int sms = 0;
      if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) sms = 152;
      s.base = static_cast<unsigned char*>(p);
      s.sm_count = sms;
      s.ready = true;
    }
    slot = s;
  }
  h.sm_count = slot.sm_count;
  if (!gspec_engine::plan_units(&h)) return fail(err, err_len, GSPEC_ERR_ARG, h.err.c_str());

  // carve the array: statistics, saturation, masks, flags, twiddles, partials
  const int N = static_cast<int>(cfg->fft_length);
  const uint64_t vals = h.dual ? 8 : 2;
  const size_t stats_b = align256(2 * gspec::kPolStats * sizeof(unsigned long long));
  const size_t sat_b = align256(h.ext_bytes);
  const size_t masks_b = align256(h.items_per_pol);
  const size_t flags_b = align256(h.batch);
  const size_t tw_b = align256(static_cast<size_t>(gspec::small_tw_size(N)) * sizeof(float2));
  const size_t part_b = h.slices > 1 ? align256(h.n_out * h.slices * vals * h.C * sizeof(float)) : 0;
  const size_t need = stats_b + sat_b + masks_b + flags_b + tw_b + part_b;
  if (need > kScratchBytes) {
    char msg[200];
    std::snprintf(msg, sizeof(msg),
                  "block needs %zu bytes of working memory, more than the %zu-byte allocation-free scratch", need,
                  kScratchBytes);
    return fail(err, err_len, GSPEC_ERR_UNSUPPORTED, msg);
  }
  unsigned char* q = slot.base;
  h.d_pol_stats = reinterpret_cast<unsigned long long*>(q);
  q += stats_b;
  unsigned long long* d_sat = reinterpret_cast<unsigned long long*>(q);
  q += sat_b;
  h.d_masks = q;
  q += masks_b;
  h.d_flags = q;
  q += flags_b;
  h.d_tw = reinterpret_cast<float2*>(q);
  q += tw_b;
  h.d_partial = part_b ? reinterpret_cast<float*>(q) : nullptr;
  h.d_baselines = d_baselines;

  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  cudaError_t e = cudaMemsetAsync(h.d_pol_stats, 0, stats_b, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(d_sat, 0, sat_b, s);
  if (e == cudaSuccess) e = gspec::launch_twiddles(N, h.d_tw, s);
  if (e == cudaSuccess)
    e = gspec_engine::run_chain(&h, static_cast<const uint8_t*>(d_block), static_cast<uint8_t*>(d_out), d_sat, s);
  if (e != cudaSuccess) return fail(err, err_len, GSPEC_ERR_CUDA, cudaGetErrorString(e));
  return GSPEC_OK;
}
