// Batch of uneven gated-spectrometer streams in one CUDA graph.
//
// Each member is an ordinary handle (its own fft_length, naccumulate, bit
// depth, pol mode and schedule).  The first gspec_batch_run captures one step
// - every member's chain over its device input block - with the members in
// parallel branches of the graph:
//
//   fork -> [phase_i -> chain_i (prepass, FFT passes, finalize) -> count_i] -> join
//
// phase_i clears member i's output accumulator when its device block counter
// starts a new output block (counter % n_blocks == 0) and count_i advances the
// counter, so the same graph serves every step of members whose n_blocks
// differ.  Each member has two input buffers and there is one graph per
// buffer; runs alternate between them, so the next step's blocks can be
// copied in while the current step runs.  Later runs replay the
// instantiated graphs with one launch each.
#include <algorithm>
#include <cstdio>
#include <string>
#include <vector>

#include "../../include/gspec.h"
#include "gspec_engine_internal.cuh"

namespace {

// out holds n_rec records of rec8 8-byte words; with one block per output
// only each record's counters (the words from spec8 on) start from zero, the
// block stores every spectrum value (gspec_engine::clear_output).
__global__ void batch_phase_kernel(const uint32_t* __restrict__ count, uint32_t n_blocks, uint2* out, uint64_t n_rec,
                                   uint64_t rec8, uint64_t spec8, uint2* sat, uint64_t n_sat8) {
  if (*count % n_blocks != 0) return;
  const uint64_t stride = static_cast<uint64_t>(gridDim.x) * blockDim.x;
  const uint64_t first = n_blocks == 1 ? spec8 : 0, per = rec8 - first;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n_rec * per; i += stride)
    out[(i / per) * rec8 + first + i % per] = make_uint2(0u, 0u);
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n_sat8; i += stride)
    sat[i] = make_uint2(0u, 0u);
}

__global__ void batch_count_kernel(uint32_t* count) { *count += 1u; }

}  // namespace

struct gspec_batch {
  int device = 0;
  int sm_count = 152;
  std::vector<gspec_handle*> h;
  uint32_t* d_count = nullptr;      // [n] blocks each member has processed
  cudaStream_t capture = nullptr;
  std::vector<cudaStream_t> branch;
  std::vector<cudaEvent_t> join;
  cudaEvent_t fork = nullptr;
  cudaGraph_t graph[2] = {nullptr, nullptr};      // one per input buffer
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  int slot = 0;                                    // input buffer the next run reads
  uint64_t kernels_per_step = 0;
  uint64_t steps = 0;
  std::string err;
};

namespace {

bool bok(gspec_batch* b, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  b->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

void batch_free(gspec_batch* b) {
  for (int i = 0; i < 2; ++i) {
    if (b->exec[i]) cudaGraphExecDestroy(b->exec[i]);
    if (b->graph[i]) cudaGraphDestroy(b->graph[i]);
  }
  for (auto* h : b->h) gspec_destroy(h);
  for (auto s : b->branch) cudaStreamDestroy(s);
  for (auto e : b->join) cudaEventDestroy(e);
  if (b->fork) cudaEventDestroy(b->fork);
  if (b->capture) cudaStreamDestroy(b->capture);
  if (b->d_count) cudaFree(b->d_count);
}

// Records one step of every member, reading input buffer `slot`, into
// b->capture (being captured).
bool record_step(gspec_batch* b, int slot) {
  if (!bok(b, cudaEventRecord(b->fork, b->capture), "fork")) return false;
  for (size_t i = 0; i < b->h.size(); ++i) {
    gspec_handle* h = b->h[i];
    cudaStream_t s = b->branch[i];
    if (!bok(b, cudaStreamWaitEvent(s, b->fork, 0), "fork wait")) return false;
    const uint64_t n8 = h->out_bytes / 8, s8 = h->ext_bytes / 8;
    const uint64_t rec8 = h->rec / 8, spec8 = (h->dual ? 8 : 2) * h->C * 4 / 8;
    const uint64_t clear8 = h->n_blocks == 1 ? h->n_out * (rec8 - spec8) : n8;
    uint64_t blocks = (std::max(clear8, s8) + 255) / 256;
    if (blocks > 4ull * b->sm_count) blocks = 4ull * b->sm_count;
    if (blocks < 1) blocks = 1;
    batch_phase_kernel<<<static_cast<unsigned>(blocks), 256, 0, s>>>(
        b->d_count + i, static_cast<uint32_t>(h->n_blocks), reinterpret_cast<uint2*>(h->d_out[0]), h->n_out, rec8,
        spec8, reinterpret_cast<uint2*>(h->d_sat[0]), s8);
    if (!bok(b, cudaGetLastError(), "phase kernel")) return false;
    if (!bok(b, gspec_engine::run_chain(h, h->d_in[slot], h->d_out[0], h->d_sat[0], s), "chain")) return false;
    batch_count_kernel<<<1, 1, 0, s>>>(b->d_count + i);
    if (!bok(b, cudaGetLastError(), "count kernel")) return false;
    if (!bok(b, cudaEventRecord(b->join[i], s), "join") ||
        !bok(b, cudaStreamWaitEvent(b->capture, b->join[i], 0), "join wait"))
      return false;
  }
  return true;
}

bool build_graph(gspec_batch* b, int slot) {
  if (!bok(b, cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), "begin capture")) return false;
  const bool rec = record_step(b, slot);
  cudaGraph_t g = nullptr;
  const cudaError_t e = cudaStreamEndCapture(b->capture, &g);
  if (!rec) {
    if (g) cudaGraphDestroy(g);
    return false;
  }
  if (!bok(b, e, "end capture")) return false;
  b->graph[slot] = g;
  size_t n = 0;
  if (!bok(b, cudaGraphGetNodes(g, nullptr, &n), "graph nodes")) return false;
  std::vector<cudaGraphNode_t> nodes(n);
  if (n && !bok(b, cudaGraphGetNodes(g, nodes.data(), &n), "graph nodes")) return false;
  b->kernels_per_step = 0;
  for (auto node : nodes) {
    cudaGraphNodeType t;
    if (cudaGraphNodeGetType(node, &t) == cudaSuccess && t == cudaGraphNodeTypeKernel) ++b->kernels_per_step;
  }
  return bok(b, cudaGraphInstantiate(&b->exec[slot], g, 0), "instantiate");
}

}  // namespace

extern "C" {

gspec_batch* gspec_batch_create(const gspec_config* cfgs, int n, char* err, size_t err_len) {
  auto report = [&](const std::string& m) {
    if (err && err_len) std::snprintf(err, err_len, "%s", m.c_str());
  };
  if (!cfgs || n <= 0) {
    report("no member configurations");
    return nullptr;
  }
  auto* b = new gspec_batch();
  b->device = cfgs[0].device;
  auto bail = [&](const std::string& m) -> gspec_batch* {
    report(m);
    batch_free(b);
    delete b;
    return nullptr;
  };
  if (cudaSetDevice(b->device) != cudaSuccess) return bail("cudaSetDevice failed");
  cudaDeviceProp prop{};
  if (cudaGetDeviceProperties(&prop, b->device) == cudaSuccess) b->sm_count = prop.multiProcessorCount;
  for (int i = 0; i < n; ++i) {
    if (cfgs[i].device != b->device) return bail("all members must use the same device");
    gspec_config c = cfgs[i];
    c.flags |= GSPEC_FLAG_NO_HOST_BUFFERS;
    char msg[256] = {0};
    gspec_handle* h = gspec_create(&c, msg, sizeof(msg));
    if (!h) return bail("member " + std::to_string(i) + ": " + msg);
    b->h.push_back(h);
    cudaStream_t s;
    if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return bail("stream");
    b->branch.push_back(s);
    cudaEvent_t e;
    if (cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return bail("event");
    b->join.push_back(e);
  }
  if (cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming) != cudaSuccess)
    return bail("stream/event");
  if (cudaMalloc(reinterpret_cast<void**>(&b->d_count), n * sizeof(uint32_t)) != cudaSuccess ||
      cudaMemset(b->d_count, 0, n * sizeof(uint32_t)) != cudaSuccess)
    return bail("block counters");
  if (cudaDeviceSynchronize() != cudaSuccess) return bail("setup");
  return b;
}

void gspec_batch_destroy(gspec_batch* b) {
  if (!b) return;
  cudaSetDevice(b->device);
  cudaDeviceSynchronize();
  batch_free(b);
  delete b;
}

int gspec_batch_size(const gspec_batch* b) { return b ? static_cast<int>(b->h.size()) : 0; }

int gspec_batch_get_info(const gspec_batch* b, int i, gspec_info* info) {
  if (!b || i < 0 || i >= static_cast<int>(b->h.size())) return GSPEC_ERR_ARG;
  return gspec_get_info(b->h[i], info);
}

void* gspec_batch_input(gspec_batch* b, int i) {
  if (!b || i < 0 || i >= static_cast<int>(b->h.size())) return nullptr;
  return b->h[i]->d_in[b->slot];
}

int gspec_batch_set_input(gspec_batch* b, int i, const void* src, size_t bytes, void* cuda_stream) {
  if (!b || !src || i < 0 || i >= static_cast<int>(b->h.size())) return GSPEC_ERR_ARG;
  gspec_handle* h = b->h[i];
  if (bytes != h->cfg.buffer_size) {
    b->err = "member " + std::to_string(i) + ": block of " + std::to_string(bytes) + " bytes, expected " +
             std::to_string(h->cfg.buffer_size);
    return GSPEC_STOP;
  }
  return bok(b, cudaMemcpyAsync(h->d_in[b->slot], src, bytes, cudaMemcpyDefault, static_cast<cudaStream_t>(cuda_stream)),
             "input copy")
             ? GSPEC_OK
             : GSPEC_ERR_CUDA;
}

int gspec_batch_read_output(gspec_batch* b, int i, void* dst, size_t bytes, void* cuda_stream) {
  if (!b || !dst || i < 0 || i >= static_cast<int>(b->h.size())) return GSPEC_ERR_ARG;
  gspec_handle* h = b->h[i];
  if (bytes > h->out_bytes) return GSPEC_ERR_ARG;
  cudaStream_t s = static_cast<cudaStream_t>(cuda_stream);
  if (!bok(b, cudaMemcpyAsync(dst, h->d_out[0], bytes, cudaMemcpyDefault, s), "output copy") ||
      !bok(b, cudaStreamSynchronize(s), "output copy"))
    return GSPEC_ERR_CUDA;
  return GSPEC_OK;
}

int gspec_batch_copy_output(gspec_batch* b, int i, void* dst, size_t bytes, void* cuda_stream) {
  if (!b || !dst || i < 0 || i >= static_cast<int>(b->h.size())) return GSPEC_ERR_ARG;
  gspec_handle* h = b->h[i];
  if (bytes > h->out_bytes) return GSPEC_ERR_ARG;
  return bok(b, cudaMemcpyAsync(dst, h->d_out[0], bytes, cudaMemcpyDefault, static_cast<cudaStream_t>(cuda_stream)),
             "output copy")
             ? GSPEC_OK
             : GSPEC_ERR_CUDA;
}

int gspec_batch_output(gspec_batch* b, int i, void** d_out, uint64_t* bytes, int* complete) {
  if (!b || i < 0 || i >= static_cast<int>(b->h.size())) return GSPEC_ERR_ARG;
  gspec_handle* h = b->h[i];
  if (d_out) *d_out = h->d_out[0];
  if (bytes) *bytes = h->out_bytes;
  if (complete) *complete = (b->steps > 0 && b->steps % h->n_blocks == 0) ? 1 : 0;
  return GSPEC_OK;
}

int gspec_batch_run(gspec_batch* b, void* cuda_stream) {
  if (!b) return GSPEC_ERR_ARG;
  if (cudaSetDevice(b->device) != cudaSuccess) return GSPEC_ERR_CUDA;
  for (auto* h : b->h)
    if (h->h_err && *h->h_err) {
      b->err = "a bounded device wait gave up (code " + std::to_string(*h->h_err) + ")";
      return GSPEC_ERR_CUDA;
    }
  if (!b->exec[b->slot] && !build_graph(b, b->slot)) return GSPEC_ERR_CUDA;
  if (!bok(b, cudaGraphLaunch(b->exec[b->slot], static_cast<cudaStream_t>(cuda_stream)), "graph launch"))
    return GSPEC_ERR_CUDA;
  b->slot ^= 1;
  ++b->steps;
  return GSPEC_OK;
}

uint64_t gspec_batch_kernels_per_step(const gspec_batch* b) { return b ? b->kernels_per_step : 0; }
uint64_t gspec_batch_steps(const gspec_batch* b) { return b ? b->steps : 0; }
const char* gspec_batch_last_error(const gspec_batch* b) { return b ? b->err.c_str() : "null batch"; }

}  // extern "C"
