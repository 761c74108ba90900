// VLBI: 8/12-bit EDD samples to 2-bit VDIF frames on the GPU, replacing
// psrdada_cpp's VLBI<Handler> (psrdada_cpp/effelsberg/edd/VLBI.cuh:91-170,
// edd/detail/VLBI.cu, edd/src/VLBI.cu).
//
// Per input block (the whole block is packed samples):
//  * vlbi_stats_kernel: exact integer sum and sum of squares of the unpacked
//    samples; mean = sum / n and sigma^2 = sum_sq / n - mean^2 in FP64 (the
//    reference sums floats in a nondeterministic order,
//    edd/detail/VLBI.cu:216-237 with edd/src/Tools.cu:8-63);
//  * vlbi_frames_kernel: every payload byte of the block's VDIF frames
//    from four samples: level = (x - mean >= -v sigma) + (x - mean >= 0) +
//    (x - mean >= v sigma), sample j of a byte in bits 2j..2j+1
//    (pack2bit_nonLinear, edd/src/VLBI.cu:183-237); the stream of a call is
//    [spill of the previous block | this block's bytes after the first-second
//    skip]; whole frames go out, the rest is the next spill
//    (edd/detail/VLBI.cu:262-318); every frame's 32-byte header is the
//    template with its frame number, second and validity (:320-350).
// The handler receives a fixed-size buffer of frames_per_block + 1 frames,
// the frames without data marked invalid, with the reference's pipeline
// delay (block n's frames at call n + 3).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <ctime>
#include <string>

#include "../../include/gspec.h"

struct gspec_vlbi {
  gspec_vlbi_config cfg{};
  std::string err;
  uint64_t nsamples = 0, packed_bytes = 0, frame_bytes = 0, payload = 0, nframes_out = 0, out_bytes = 0;
  uint64_t bytes_to_skip = 0, spill = 0;
  uint32_t header[8] = {0};           // the running header: next frame's number and second
  uint64_t frames_per_second = 0;
  int call_count = 0;
  int ia = 0;
  uint8_t* d_in[2] = {nullptr, nullptr};
  uint8_t* d_out[2] = {nullptr, nullptr};
  uint8_t* d_spill[2] = {nullptr, nullptr};   // spill-over bytes, double-buffered (read old, write new)
  unsigned long long* d_stats = nullptr;      // [sum, sum of squares]
  char* h_out[2] = {nullptr, nullptr};
  cudaStream_t h2d = nullptr, proc = nullptr, d2h = nullptr;
  cudaEvent_t ev_h2d[2] = {nullptr, nullptr}, ev_in_free[2] = {nullptr, nullptr}, ev_out[2] = {nullptr, nullptr};
  int si = 0;                                  // spill buffer holding the current spill
  double last_mean = 0.0, last_sigma = 0.0;
  unsigned long long* h_stats = nullptr;       // pinned copy of the last block's sums
};

namespace {

__device__ __forceinline__ int sample_at(const uint8_t* __restrict__ b, uint32_t nbits, uint64_t i) {
  if (nbits == 8) return static_cast<int8_t>(b[i]);
  // 12 bit: two samples per 3 bytes, big-endian, MSB first
  const uint64_t byte = (i >> 1) * 3;
  const uint32_t w = (static_cast<uint32_t>(b[byte]) << 16) | (static_cast<uint32_t>(b[byte + 1]) << 8) | b[byte + 2];
  const uint32_t v = (i & 1) ? (w & 0xFFF) : (w >> 12);
  return static_cast<int>(v << 20) >> 20;
}

__global__ void vlbi_stats_kernel(const uint8_t* __restrict__ in, uint32_t nbits, uint64_t n,
                                  unsigned long long* stats) {
  long long s = 0;
  unsigned long long q = 0;
  for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
       i += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    const int v = sample_at(in, nbits, i);
    s += v;
    q += static_cast<unsigned long long>(v * v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    s += __shfl_xor_sync(0xffffffffu, s, o);
    q += __shfl_xor_sync(0xffffffffu, q, o);
  }
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(stats, static_cast<unsigned long long>(s));
    atomicAdd(stats + 1, q);
  }
}

struct FrameParams {
  const uint8_t* in;
  const uint8_t* spill_in;
  uint8_t* spill_out;
  uint8_t* out;
  const unsigned long long* stats;
  uint64_t nsamples;        // samples of the block
  uint64_t skip;            // bytes of this block's 2-bit stream skipped (first-second alignment)
  uint64_t spill;           // bytes carried in from the previous block
  uint64_t payload, frame_bytes, nvalid, nframes;
  uint64_t new_spill;
  uint32_t nbits;
  float v;                  // digitizer threshold in units of sigma
  uint32_t header[8];       // template of frame 0 (its number and second)
  uint64_t frames_per_second;
};

__device__ __forceinline__ uint32_t set_bits(uint32_t w, int first, int last, uint32_t v) {
  const uint32_t mask = (last - first == 31) ? 0xFFFFFFFFu : (((1u << (last - first + 1)) - 1u) << first);
  return (w & ~mask) | ((v << first) & mask);
}

// 2-bit level of sample x with the block statistics (pack2bit_nonLinear)
__device__ __forceinline__ uint32_t level2(int x, float mean, float vsigma) {
  const float inp = __fsub_rn(static_cast<float>(x), mean);
  const double d = inp, t = vsigma;
  return (d >= -t) + (d >= 0.0) + (d >= t);
}

__global__ void vlbi_frames_kernel(FrameParams p) {
  const double n = static_cast<double>(p.nsamples);
  const double mean_d = static_cast<double>(static_cast<long long>(p.stats[0])) / n;
  const double var = static_cast<double>(p.stats[1]) / n - mean_d * mean_d;
  const float mean = static_cast<float>(mean_d);
  const float vsigma = __fmul_rn(p.v, sqrtf(static_cast<float>(var > 0.0 ? var : 0.0)));
  const uint64_t total = p.nframes * p.frame_bytes;
  const uint64_t stream_bytes = p.nvalid * p.payload + p.new_spill;   // bytes of this call's stream used
  for (uint64_t o = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; o < total + p.new_spill;
       o += static_cast<uint64_t>(gridDim.x) * blockDim.x) {
    uint64_t q;          // position in the call's stream
    uint8_t* dst;
    if (o < total) {
      const uint64_t f = o / p.frame_bytes, b = o - f * p.frame_bytes;
      if (b < 32) {
        if ((b & 3) == 0) {
          // header word b / 4 of frame f
          const int w = static_cast<int>(b >> 2);
          uint32_t val = p.header[w];
          if (w == 0 || w == 1) {
            const uint64_t num = (p.header[1] & 0xFFFFFFu) + f;
            const uint64_t sec = (p.header[0] & 0x3FFFFFFFu) + num / p.frames_per_second;
            if (w == 0) {
              val = set_bits(val, 0, 29, static_cast<uint32_t>(sec));
              val = set_bits(val, 31, 31, f < p.nvalid ? 0u : 1u);   // bit 31: invalid
            } else {
              val = set_bits(val, 0, 23, static_cast<uint32_t>(num % p.frames_per_second));
            }
          }
          *reinterpret_cast<uint32_t*>(p.out + o) = val;
        }
        continue;
      }
      if (f >= p.nvalid) {
        p.out[o] = 0;
        continue;
      }
      q = f * p.payload + (b - 32);
      dst = p.out + o;
    } else {
      q = p.nvalid * p.payload + (o - total);   // the new spill
      dst = p.spill_out + (o - total);
    }
    if (q >= stream_bytes) continue;
    if (q < p.spill) {
      *dst = p.spill_in[q];
      continue;
    }
    const uint64_t i = (q - p.spill + p.skip) * 4;   // first sample of the byte
    uint32_t byte = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) byte |= level2(sample_at(p.in, p.nbits, i + j), mean, vsigma) << (2 * j);
    *dst = static_cast<uint8_t>(byte);
  }
}

int set_err(gspec_vlbi* h, int code, const std::string& m) {
  if (h) h->err = m;
  return code;
}

bool ok(gspec_vlbi* h, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  h->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

// days from 1970-01-01 of a proleptic Gregorian date (Howard Hinnant's days_from_civil)
long long days_from_civil(long long y, unsigned m, unsigned d) {
  y -= m <= 2;
  const long long era = (y >= 0 ? y : y - 399) / 400;
  const unsigned yoe = static_cast<unsigned>(y - era * 400);
  const unsigned doy = (153 * (m + (m > 2 ? -3 : 9)) + 2) / 5 + d - 1;
  const unsigned doe = yoe * 365 + yoe / 4 - yoe / 100 + doy;
  return era * 146097 + static_cast<long long>(doe) - 719468;
}

void release(gspec_vlbi* h) {
  for (int i = 0; i < 2; ++i) {
    cudaFree(h->d_in[i]);
    cudaFree(h->d_out[i]);
    cudaFree(h->d_spill[i]);
    if (h->h_out[i]) cudaFreeHost(h->h_out[i]);
    if (h->ev_h2d[i]) cudaEventDestroy(h->ev_h2d[i]);
    if (h->ev_in_free[i]) cudaEventDestroy(h->ev_in_free[i]);
    if (h->ev_out[i]) cudaEventDestroy(h->ev_out[i]);
  }
  cudaFree(h->d_stats);
  if (h->h_stats) cudaFreeHost(h->h_stats);
  if (h->h2d) cudaStreamDestroy(h->h2d);
  if (h->proc) cudaStreamDestroy(h->proc);
  if (h->d2h) cudaStreamDestroy(h->d2h);
}

}  // namespace

extern "C" {

int gspec_vdif_set_time(uint32_t* header, uint64_t posix_seconds) {
  if (!header) return GSPEC_ERR_ARG;
  // VDIF reference epoch: half-years since 2000-01-01 (the epoch starts on 1 Jan or 1 Jul UTC)
  const long long days = static_cast<long long>(posix_seconds / 86400);
  // civil date from days (inverse of days_from_civil)
  const long long z = days + 719468;
  const long long era = (z >= 0 ? z : z - 146096) / 146097;
  const unsigned doe = static_cast<unsigned>(z - era * 146097);
  const unsigned yoe = (doe - doe / 1460 + doe / 36524 - doe / 146096) / 365;
  const unsigned doy = doe - (365 * yoe + yoe / 4 - yoe / 100);
  const unsigned mp = (5 * doy + 2) / 153;
  const unsigned m = mp < 10 ? mp + 3 : mp - 9;
  const long long y = static_cast<long long>(yoe) + era * 400 + (m <= 2);
  if (y < 2000) return GSPEC_ERR_ARG;    // VDIF cannot encode times before 2000
  const unsigned half = m >= 7 ? 1u : 0u;
  const long long epoch_start = days_from_civil(y, half ? 7 : 1, 1) * 86400;
  const uint32_t ref_epoch = static_cast<uint32_t>((y - 2000) * 2 + half);
  header[1] = (header[1] & ~(0x3Fu << 24)) | ((ref_epoch & 0x3Fu) << 24);
  header[0] = (header[0] & ~0x3FFFFFFFu) | (static_cast<uint32_t>(posix_seconds - epoch_start) & 0x3FFFFFFFu);
  return GSPEC_OK;
}

gspec_vlbi* gspec_vlbi_create(const gspec_vlbi_config* cfg, char* err, size_t err_len) {
  auto fail = [&](const std::string& m) -> gspec_vlbi* {
    if (err && err_len) std::snprintf(err, err_len, "%s", m.c_str());
    return nullptr;
  };
  if (!cfg) return fail("null configuration");
  if (cfg->nbits != 8 && cfg->nbits != 12) return fail("nbits must be 8 or 12");
  if (cfg->buffer_size == 0 || (cfg->buffer_size * 8) % cfg->nbits) return fail("buffer holds no whole samples");
  const uint64_t frame_len = cfg->vdif_header[2] & 0xFFFFFFu;   // 8-byte units, header included
  if (frame_len * 8 <= 32) return fail("the VDIF header template needs a data frame length above 32 bytes");
  if (!(cfg->sample_rate > 0.0) || !(cfg->digitizer_threshold > 0.0)) return fail("sample rate and threshold > 0");
  auto* h = new gspec_vlbi();
  h->cfg = *cfg;
  h->nsamples = cfg->buffer_size * 8 / cfg->nbits;
  if (h->nsamples % 4) {
    delete h;
    return fail("samples per block must be a multiple of 4 (whole 2-bit bytes)");
  }
  h->packed_bytes = h->nsamples / 4;
  h->frame_bytes = frame_len * 8;
  h->payload = h->frame_bytes - 32;
  h->nframes_out = h->packed_bytes / h->payload + 1;
  h->out_bytes = h->nframes_out * h->frame_bytes;
  std::memcpy(h->header, cfg->vdif_header, sizeof(h->header));
  // 2 bits per sample (bits/sample - 1 = 1), real data (edd/detail/VLBI.cu:84-85)
  h->header[3] = (h->header[3] & ~(0x1Fu << 26)) | (1u << 26);
  h->header[3] &= ~(1u << 31);
  const uint64_t samples_per_frame = h->payload * 4;
  h->frames_per_second = static_cast<uint64_t>(cfg->sample_rate / static_cast<double>(samples_per_frame));
  if (h->frames_per_second == 0) {
    delete h;
    return fail("fewer than one VDIF frame per second at this sample rate");
  }
  if (cudaSetDevice(cfg->device) != cudaSuccess) {
    delete h;
    return fail("cudaSetDevice failed");
  }
  bool good = ok(h, cudaStreamCreateWithFlags(&h->h2d, cudaStreamNonBlocking), "stream") &&
              ok(h, cudaStreamCreateWithFlags(&h->proc, cudaStreamNonBlocking), "stream") &&
              ok(h, cudaStreamCreateWithFlags(&h->d2h, cudaStreamNonBlocking), "stream") &&
              ok(h, cudaMalloc(&h->d_stats, 2 * sizeof(unsigned long long)), "stats") &&
              ok(h, cudaMallocHost(&h->h_stats, 2 * sizeof(unsigned long long)), "stats");
  for (int i = 0; good && i < 2; ++i)
    good = ok(h, cudaMalloc(&h->d_in[i], cfg->buffer_size), "input") &&
           ok(h, cudaMalloc(&h->d_out[i], h->out_bytes), "frames") &&
           ok(h, cudaMalloc(&h->d_spill[i], h->payload), "spill") &&
           ok(h, cudaMallocHost(reinterpret_cast<void**>(&h->h_out[i]), h->out_bytes), "host frames") &&
           ok(h, cudaEventCreateWithFlags(&h->ev_h2d[i], cudaEventDisableTiming), "event") &&
           ok(h, cudaEventCreateWithFlags(&h->ev_in_free[i], cudaEventDisableTiming), "event") &&
           ok(h, cudaEventCreateWithFlags(&h->ev_out[i], cudaEventDisableTiming), "event");
  if (!good) {
    const std::string m = h->err;
    release(h);
    delete h;
    return fail(m);
  }
  return h;
}

void gspec_vlbi_destroy(gspec_vlbi* h) {
  if (!h) return;
  cudaSetDevice(h->cfg.device);
  if (h->h2d) cudaStreamSynchronize(h->h2d);
  if (h->proc) cudaStreamSynchronize(h->proc);
  if (h->d2h) cudaStreamSynchronize(h->d2h);
  release(h);
  delete h;
}

const char* gspec_vlbi_last_error(gspec_vlbi* h) { return h ? h->err.c_str() : "null handle"; }

// edd/detail/VLBI.cu:92-134: time of the first sample from SYNC_TIME and
// SAMPLE_CLOCK_START; VDIF starts on the next whole second, the samples
// before it are skipped; the header's epoch and second are set from it; the
// line "# VLBI parameters:" is appended to the header when it fits.
int gspec_vlbi_init(gspec_vlbi* h, char* header, size_t total_bytes) {
  if (!h || !header) return GSPEC_ERR_ARG;
  const size_t end = strnlen(header, total_bytes);
  const std::string text(header, end);
  auto value = [&](const char* key, long long& out) {
    // one "KEY value" line (ascii_header_get semantics: key at a line start)
    size_t pos = 0;
    int found = 0;
    while ((pos = text.find(key, pos)) != std::string::npos) {
      const bool line_start = pos == 0 || text[pos - 1] == '\n';
      const size_t after = pos + std::strlen(key);
      if (line_start && after < text.size() && (text[after] == ' ' || text[after] == '\t')) {
        out = std::strtoll(text.c_str() + after, nullptr, 10);
        ++found;
      }
      pos = after;
    }
    return found == 1;
  };
  long long sync_time = 0, clock_start = 0;
  if (!value("SYNC_TIME", sync_time) || !value("SAMPLE_CLOCK_START", clock_start)) {
    h->err = "No or multiple SYNC_TIME / SAMPLE_CLOCK_START in the header: the time reference is not set";
    return GSPEC_STOP;
  }
  const double frac = static_cast<double>(sync_time) + static_cast<double>(clock_start) / h->cfg.sample_rate;
  const uint64_t ts = static_cast<uint64_t>(frac) + 1;
  const uint64_t samples_to_skip = static_cast<uint64_t>((static_cast<double>(ts) - frac) * h->cfg.sample_rate);
  h->bytes_to_skip = samples_to_skip * 2 / 8;
  if (gspec_vdif_set_time(h->header, ts) != GSPEC_OK) {
    h->err = "Cannot encode a time before 1 Jan 2000 in VDIF";
    return GSPEC_ERR_ARG;
  }
  static const char kInfo[] = "\n# VLBI parameters: \n";
  if (end + sizeof(kInfo) - 1 < total_bytes) std::memcpy(header + end, kInfo, sizeof(kInfo));
  return GSPEC_OK;
}

int gspec_vlbi_process(gspec_vlbi* h, const char* block, size_t used, gspec_output* out) {
  if (!h || !out) return GSPEC_ERR_ARG;
  out->ready = 0;
  out->data = nullptr;
  out->size = 0;
  if (cudaSetDevice(h->cfg.device) != cudaSuccess) return set_err(h, GSPEC_ERR_CUDA, "cudaSetDevice failed");
  // whole blocks before the first VDIF second are dropped (edd/detail/VLBI.cu:142-148)
  if (h->bytes_to_skip > h->packed_bytes) {
    h->bytes_to_skip -= h->packed_bytes;
    return GSPEC_OK;
  }
  if (used != h->cfg.buffer_size)
    return set_err(h, GSPEC_STOP,
                   "Unexpected Buffer Size - Got " + std::to_string(used) + " byte, expected " +
                       std::to_string(h->cfg.buffer_size) + " byte");
  if (!block) return set_err(h, GSPEC_ERR_ARG, "null block");
  ++h->call_count;
  h->ia ^= 1;
  const int ia = h->ia, ib = ia ^ 1;
  if (!ok(h, cudaStreamWaitEvent(h->h2d, h->ev_in_free[ia], 0), "wait") ||
      !ok(h, cudaMemcpyAsync(h->d_in[ia], block, h->cfg.buffer_size, cudaMemcpyHostToDevice, h->h2d), "H2D") ||
      !ok(h, cudaEventRecord(h->ev_h2d[ia], h->h2d), "event"))
    return GSPEC_ERR_CUDA;
  // the previous call's frames copy has landed: its device buffer is free and
  // its host buffer is complete
  if (!ok(h, cudaStreamSynchronize(h->d2h), "D2H")) return GSPEC_ERR_CUDA;
  const int c = h->call_count;
  if (c >= 2) {
    // block c - 1: statistics, then its frames into device buffer c % 2
    const int oa = c & 1;
    const uint64_t stream_bytes = h->spill + h->packed_bytes - h->bytes_to_skip;
    const uint64_t nvalid = stream_bytes / h->payload;
    FrameParams p{};
    p.in = h->d_in[ib];
    p.spill_in = h->d_spill[h->si];
    p.spill_out = h->d_spill[h->si ^ 1];
    p.out = h->d_out[oa];
    p.stats = h->d_stats;
    p.nsamples = h->nsamples;
    p.skip = h->bytes_to_skip;
    p.spill = h->spill;
    p.payload = h->payload;
    p.frame_bytes = h->frame_bytes;
    p.nvalid = nvalid;
    p.nframes = h->nframes_out;
    p.new_spill = stream_bytes - nvalid * h->payload;
    p.nbits = h->cfg.nbits;
    p.v = static_cast<float>(h->cfg.digitizer_threshold);
    std::memcpy(p.header, h->header, sizeof(p.header));
    p.frames_per_second = h->frames_per_second;
    if (!ok(h, cudaStreamWaitEvent(h->proc, h->ev_h2d[ib], 0), "wait") ||
        !ok(h, cudaMemsetAsync(h->d_stats, 0, 2 * sizeof(unsigned long long), h->proc), "stats"))
      return GSPEC_ERR_CUDA;
    vlbi_stats_kernel<<<304, 256, 0, h->proc>>>(h->d_in[ib], h->cfg.nbits, h->nsamples, h->d_stats);
    vlbi_frames_kernel<<<1216, 256, 0, h->proc>>>(p);
    if (!ok(h, cudaGetLastError(), "VLBI kernels") || !ok(h, cudaEventRecord(h->ev_in_free[ib], h->proc), "event") ||
        !ok(h, cudaMemcpyAsync(h->h_stats, h->d_stats, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost,
                               h->proc),
            "stats copy") ||
        !ok(h, cudaEventRecord(h->ev_out[oa], h->proc), "event"))
      return GSPEC_ERR_CUDA;
    // the running header: frame numbers and seconds advance by the valid frames
    const uint64_t num = (h->header[1] & 0xFFFFFFu) + nvalid;
    const uint64_t sec = (h->header[0] & 0x3FFFFFFFu) + num / h->frames_per_second;
    h->header[1] = (h->header[1] & ~0xFFFFFFu) | static_cast<uint32_t>(num % h->frames_per_second);
    h->header[0] = (h->header[0] & ~0x3FFFFFFFu) | static_cast<uint32_t>(sec & 0x3FFFFFFFu);
    h->spill = p.new_spill;
    h->si ^= 1;
    h->bytes_to_skip = 0;
  }
  if (c >= 3) {
    // block c - 2's frames (computed at the previous call) to host buffer c % 2
    const int prev = (c - 1) & 1;
    if (!ok(h, cudaStreamWaitEvent(h->d2h, h->ev_out[prev], 0), "wait") ||
        !ok(h, cudaMemcpyAsync(h->h_out[c & 1], h->d_out[prev], h->out_bytes, cudaMemcpyDeviceToHost, h->d2h),
            "D2H"))
      return GSPEC_ERR_CUDA;
  }
  if (c >= 4) {
    // block c - 3's frames, copied at the previous call (complete: synchronised above)
    out->data = h->h_out[(c - 1) & 1];
    out->size = h->out_bytes;
    out->ready = 1;
  }
  if (!ok(h, cudaStreamSynchronize(h->h2d), "H2D")) return GSPEC_ERR_CUDA;
  return GSPEC_OK;
}

int gspec_vlbi_get_info(gspec_vlbi* h, gspec_vlbi_info* info) {
  if (!h || !info) return GSPEC_ERR_ARG;
  info->frame_bytes = h->frame_bytes;
  info->frames_per_output = h->nframes_out;
  info->output_bytes = h->out_bytes;
  info->frames_per_second = h->frames_per_second;
  info->bytes_to_skip = h->bytes_to_skip;
  info->spill_bytes = h->spill;
  std::memcpy(info->header, h->header, sizeof(info->header));
  info->last_sum = static_cast<long long>(h->h_stats ? h->h_stats[0] : 0);
  info->last_sum_sq = h->h_stats ? h->h_stats[1] : 0;
  return GSPEC_OK;
}

}  // extern "C"
