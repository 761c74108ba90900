// Serving loop: many concurrent gated-spectrometer streams on one GPU.
//
// The reference runs one GatedSpectrometer per process, fed by one DADA ring
// (psrdada_cpp/detail/dada_input_stream.cpp:21-52); nothing in it serves
// several streams.  Here one scheduler thread owns the GPU side of every
// admitted stream:
//   * admission: a stream is admitted when the device bytes its handle needs
//     (gspec_query) fit into the budget next to the admitted ones; waiting
//     streams are admitted in FIFO order as closed streams free memory;
//   * state: each admitted stream keeps its handle (baselines, counters,
//     output accumulators, twiddles, scratch) resident in device memory;
//   * continuous batching: a stream's next block is issued as soon as it is
//     queued, its stream has fewer than max_inflight blocks on the GPU, the
//     input bytes of long blocks (> 64 MiB) on the GPU stay within
//     inflight_bytes (short blocks are never held back) and a host output
//     buffer is free, so blocks of different streams overlap on the device in
//     their own CUDA streams (streams are scanned in id order each pass);
//   * completion: each block's last operation records an event; the loop
//     queries the oldest event of every stream and posts results in order.
// Per block the work is the handle's chain (gspec_engine::run_chain): H2D on
// the handle's copy stream (in 8 MiB pieces) into one of two input buffers,
// the chain on its compute stream into one of two output accumulators, and at
// the end of an output block the accumulator's way to the host: SM stores
// into the page-locked result buffer for outputs up to 16 MiB, else a D2H
// copy (in pieces) on the handle's copy-out stream.
#include <chrono>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gspec.h"
#include "gspec_engine_internal.cuh"

namespace {

using Clock = std::chrono::steady_clock;

struct Queued {
  const void* data;
  size_t size;
  uint64_t tag;
  uint64_t index;
  double t_submit;
};

struct Flight {
  uint64_t index;
  uint64_t tag;
  double t_submit;
  double t_start;
  int obuf;        // host output buffer, -1 when the block completes no output
  cudaEvent_t done;
  uint64_t bytes;  // input bytes of a long block (in-flight limit), else 0
  int slot;        // event slot of the stage timings
};

constexpr int kEventsPerStream = 4;

struct Stream {
  int id = 0;
  gspec_config cfg{};
  gspec_info info{};
  uint64_t bytes = 0;          // device bytes (admission)
  int state = 0;               // 0 waiting, 1 admitted, 2 closing, 3 closed, 4 being admitted, 5 being freed
  bool close_requested = false;
  gspec_handle* h = nullptr;
  std::deque<Queued> queue;
  std::deque<Flight> flight;
  uint64_t submitted = 0;
  uint64_t issued = 0;
  std::vector<char*> hbuf;
  std::vector<char*> hbuf_dev;   // device addresses of hbuf
  std::vector<int> hfree;
  cudaEvent_t ev[kEventsPerStream] = {};        // block finished
  cudaEvent_t ev_stage[4][kEventsPerStream] = {};   // copy start, copy end, chain start, chain end
  int ev_next = 0;
  cudaEvent_t ev_out_done[2] = {};   // D2H of output accumulator i finished
  cudaEvent_t ev_out_full[2] = {};   // chain of the last block of output i finished
  bool failed = false;
};

}  // namespace

struct gspec_server {
  gspec_server_config cfg{};
  Clock::time_point t0;
  mutable std::mutex mu;
  std::condition_variable cv_work;
  std::condition_variable cv_result;
  std::vector<std::unique_ptr<Stream>> streams;
  std::deque<int> admit;
  std::deque<gspec_result> results;
  uint64_t in_use = 0;
  uint64_t inflight_bytes = 0;  // input bytes of the long blocks on the GPU
  uint64_t launches_done = 0;   // launches of streams already closed
  cudaEvent_t epoch = nullptr;  // GPU time of server-clock second t_epoch
  double t_epoch = 0;
  bool stop = false;
  std::thread worker;
  std::string err;
};

namespace {

double now_s(const gspec_server* s) {
  return std::chrono::duration<double>(Clock::now() - s->t0).count();
}

bool ok(Stream& st, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  st.failed = true;
  if (st.h) st.h->err = std::string(what) + ": " + cudaGetErrorString(e);
  return false;
}

void free_stream_memory(Stream& st) {
  for (char* p : st.hbuf)
    if (p) cudaFreeHost(p);
  st.hbuf.clear();
  st.hbuf_dev.clear();
  st.hfree.clear();
  for (auto& e : st.ev)
    if (e) cudaEventDestroy(e), e = nullptr;
  for (auto& row : st.ev_stage)
    for (auto& e : row)
      if (e) cudaEventDestroy(e), e = nullptr;
  for (int i = 0; i < 2; ++i) {
    if (st.ev_out_done[i]) cudaEventDestroy(st.ev_out_done[i]), st.ev_out_done[i] = nullptr;
    if (st.ev_out_full[i]) cudaEventDestroy(st.ev_out_full[i]), st.ev_out_full[i] = nullptr;
  }
  if (st.h) gspec_destroy(st.h);
  st.h = nullptr;
}

// Moves the GPU resources (handle, events, host buffers) from src to dst.
void take_resources(Stream& dst, Stream& src) {
  dst.h = src.h;
  src.h = nullptr;
  dst.info = src.info;
  dst.hbuf.swap(src.hbuf);
  dst.hbuf_dev.swap(src.hbuf_dev);
  dst.hfree.swap(src.hfree);
  for (int i = 0; i < kEventsPerStream; ++i) {
    std::swap(dst.ev[i], src.ev[i]);
    for (int k = 0; k < 4; ++k) std::swap(dst.ev_stage[k][i], src.ev_stage[k][i]);
  }
  for (int i = 0; i < 2; ++i) {
    std::swap(dst.ev_out_done[i], src.ev_out_done[i]);
    std::swap(dst.ev_out_full[i], src.ev_out_full[i]);
  }
}

// Creates the handle and host buffers of an admitted stream into st (called
// by the worker without the server lock: pinning host memory and allocating
// device memory take milliseconds to seconds).
bool admit_stream(const gspec_server_config& scfg, const gspec_config& cfg, int id, Stream& st, std::string& err) {
  char msg[256] = {0};
  gspec_config c = cfg;
  c.device = scfg.device;
  c.flags |= GSPEC_FLAG_NO_HOST_BUFFERS;
  st.h = gspec_create(&c, msg, sizeof(msg));
  if (!st.h) {
    err = std::string("stream ") + std::to_string(id) + ": " + msg;
    return false;
  }
  gspec_get_info(st.h, &st.info);
  const int nb = scfg.output_buffers > 0 ? scfg.output_buffers : 2;
  st.hbuf.assign(nb, nullptr);
  st.hbuf_dev.assign(nb, nullptr);
  st.hfree.assign(nb, 1);
  for (int i = 0; i < nb; ++i)
    if (cudaMallocHost(reinterpret_cast<void**>(&st.hbuf[i]), st.info.output_bytes) != cudaSuccess ||
        cudaHostGetDevicePointer(reinterpret_cast<void**>(&st.hbuf_dev[i]), st.hbuf[i], 0) != cudaSuccess)
      return false;
  for (auto& e : st.ev)
    if (cudaEventCreate(&e) != cudaSuccess) return false;
  for (auto& row : st.ev_stage)
    for (auto& e : row)
      if (cudaEventCreate(&e) != cudaSuccess) return false;
  for (int i = 0; i < 2; ++i) {
    if (cudaEventCreateWithFlags(&st.ev_out_done[i], cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&st.ev_out_full[i], cudaEventDisableTiming) != cudaSuccess)
      return false;
    // nothing to wait for before the first use of either accumulator
    cudaEventRecord(st.ev_out_done[i], st.h->d2h);
  }
  return true;
}

// Large copies go out in pieces: the copy engines take work from the streams
// of all served streams piece by piece, so a short block's copy waits for at
// most one piece of a long block's copy instead of the whole of it.
#ifndef GSPEC_COPY_PIECE_MB
#define GSPEC_COPY_PIECE_MB 8
#endif
constexpr size_t kCopyPiece = static_cast<size_t>(GSPEC_COPY_PIECE_MB) << 20;

cudaError_t copy_pieces(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t s) {
  auto* d = static_cast<char*>(dst);
  auto* p = static_cast<const char*>(src);
  for (size_t off = 0; off < bytes; off += kCopyPiece) {
    const size_t n = bytes - off < kCopyPiece ? bytes - off : kCopyPiece;
    const cudaError_t e = cudaMemcpyAsync(d + off, p + off, n, kind, s);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// Short blocks (inputs up to kShortBlockMax) and outputs up to kStoreCopyMax
// move between page-locked host memory and the GPU by SM loads and stores on
// the compute stream: the copy engines take copies in the order they were
// issued, so a short block's copy would otherwise wait behind every long
// block's copy issued before it.  Short blocks are never held back by the
// server's in-flight limit either.
constexpr uint64_t kShortBlockMax = 64u << 20;
constexpr uint64_t kStoreCopyMax = 16u << 20;

// Device address of a page-locked host block, or nullptr (pageable memory,
// device memory) when the block goes through the copy engines.
const void* mapped_host(const void* p) {
  cudaPointerAttributes a{};
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// Enqueues one block of an admitted stream on its handle's streams.
bool issue(gspec_server* s, Stream& st, const Queued& q, int obuf) {
  gspec_handle* h = st.h;
  const int slot = static_cast<int>(st.issued & 1);
  const uint64_t nb = st.info.n_blocks;
  const int oi = static_cast<int>((q.index / nb) & 1);
  const bool first = q.index % nb == 0;
  const bool last = obuf >= 0;
  const int es = st.ev_next;
  Flight f{q.index, q.tag, q.t_submit, now_s(s), obuf, st.ev[es], q.size > kShortBlockMax ? q.size : 0, es};
  st.ev_next = (st.ev_next + 1) % kEventsPerStream;
  const bool words = q.size % 8 == 0 && reinterpret_cast<uintptr_t>(q.data) % 8 == 0;
  const void* src_dev = q.size <= kShortBlockMax && words ? mapped_host(q.data) : nullptr;
  if (src_dev) {
    // the compute stream's earlier chains are the input slot's only readers
    if (!ok(st, cudaEventRecord(st.ev_stage[0][es], h->proc), "record") ||
        !ok(st, gspec::launch_copy_words(h->d_in[slot], src_dev, q.size, h->sm_count, h->proc), "input copy") ||
        !ok(st, cudaEventRecord(st.ev_stage[1][es], h->proc), "record"))
      return false;
    h->launches += 1;
  } else if (!ok(st, cudaStreamWaitEvent(h->h2d, h->ev_in_free[slot], 0), "wait input") ||
             !ok(st, cudaEventRecord(st.ev_stage[0][es], h->h2d), "record") ||
             !ok(st, copy_pieces(h->d_in[slot], q.data, q.size, cudaMemcpyDefault, h->h2d), "H2D block") ||
             !ok(st, cudaEventRecord(h->ev_h2d[slot], h->h2d), "record") ||
             !ok(st, cudaEventRecord(st.ev_stage[1][es], h->h2d), "record") ||
             !ok(st, cudaStreamWaitEvent(h->proc, h->ev_h2d[slot], 0), "wait H2D")) {
    return false;
  }
  if (first) {
    // the accumulator's previous D2H must be done before it is cleared
    if (!ok(st, cudaStreamWaitEvent(h->proc, st.ev_out_done[oi], 0), "wait D2H") ||
        !ok(st, gspec_engine::clear_output(h, h->d_out[oi], h->proc), "clear output") ||
        !ok(st, cudaMemsetAsync(h->d_sat[oi], 0, h->ext_bytes, h->proc), "clear saturation"))
      return false;
  }
  if (!ok(st, cudaEventRecord(st.ev_stage[2][es], h->proc), "record") ||
      !ok(st, gspec_engine::run_chain(h, h->d_in[slot], h->d_out[oi], h->d_sat[oi], h->proc), "chain") ||
      !ok(st, cudaEventRecord(h->ev_in_free[slot], h->proc), "record") ||
      !ok(st, cudaEventRecord(st.ev_stage[3][es], h->proc), "record"))
    return false;
  const bool sat = (st.cfg.flags & GSPEC_FLAG_SATURATION_RECORD) != 0;
  if (last && h->out_bytes + (sat ? h->ext_bytes : 0) <= kStoreCopyMax) {
    char* dst = st.hbuf_dev[obuf];
    if (!ok(st, gspec::launch_copy_words(dst, h->d_out[oi], h->out_bytes, h->sm_count, h->proc), "output copy") ||
        (sat && !ok(st, gspec::launch_copy_words(dst + h->out_bytes, h->d_sat[oi], h->ext_bytes, h->sm_count, h->proc),
                    "saturation copy")) ||
        !ok(st, cudaEventRecord(st.ev_out_done[oi], h->proc), "record") ||
        !ok(st, cudaEventRecord(f.done, h->proc), "record"))
      return false;
    h->launches += sat ? 2 : 1;
  } else if (last) {
    char* dst = st.hbuf[obuf];
    if (!ok(st, cudaEventRecord(st.ev_out_full[oi], h->proc), "record") ||
        !ok(st, cudaStreamWaitEvent(h->d2h, st.ev_out_full[oi], 0), "wait output") ||
        !ok(st, copy_pieces(dst, h->d_out[oi], h->out_bytes, cudaMemcpyDeviceToHost, h->d2h), "D2H output"))
      return false;
    if (sat && !ok(st, cudaMemcpyAsync(dst + h->out_bytes, h->d_sat[oi], h->ext_bytes, cudaMemcpyDeviceToHost, h->d2h),
            "D2H saturation"))
      return false;
    if (!ok(st, cudaEventRecord(st.ev_out_done[oi], h->d2h), "record") ||
        !ok(st, cudaEventRecord(f.done, h->d2h), "record"))
      return false;
  } else {
    if (!ok(st, cudaEventRecord(f.done, h->proc), "record")) return false;
  }
  ++st.issued;
  s->inflight_bytes += f.bytes;
  st.flight.push_back(f);
  return true;
}

gspec_result make_result(const gspec_server* s, const Stream& st, const Flight& f, int status, double t_done) {
  gspec_result r{};
  r.stream = st.id;
  r.status = status;
  r.tag = f.tag;
  r.block_index = f.index;
  r.data = f.obuf >= 0 ? st.hbuf[f.obuf] : nullptr;
  r.size = f.obuf >= 0 ? st.info.output_bytes : 0;
  r.buffer = f.obuf;
  r.t_submit = f.t_submit;
  r.t_start = f.t_start;
  r.t_done = t_done;
  if (f.done && f.slot >= 0 && status == GSPEC_OK) {
    auto ms = [](cudaEvent_t a, cudaEvent_t b) {
      float v = 0.f;
      return cudaEventElapsedTime(&v, a, b) == cudaSuccess ? v : -1.f;
    };
    r.h2d_ms = ms(st.ev_stage[0][f.slot], st.ev_stage[1][f.slot]);
    r.wait_ms = ms(st.ev_stage[1][f.slot], st.ev_stage[2][f.slot]);
    r.chain_ms = ms(st.ev_stage[2][f.slot], st.ev_stage[3][f.slot]);
    r.d2h_ms = ms(st.ev_stage[3][f.slot], f.done);
    if (s->epoch) {
      const float g0 = ms(s->epoch, st.ev_stage[0][f.slot]), g1 = ms(s->epoch, f.done);
      if (g0 >= 0.f) r.issue_ms = static_cast<float>((s->t_epoch + g0 * 1e-3 - f.t_start) * 1e3);
      if (g1 >= 0.f) r.observe_ms = static_cast<float>((t_done - s->t_epoch - g1 * 1e-3) * 1e3);
    }
  }
  return r;
}

bool stream_idle(const Stream& st) {
  if (!st.queue.empty() || !st.flight.empty()) return false;
  for (int f : st.hfree)
    if (!f) return false;
  return true;
}

void worker_loop(gspec_server* s) {
  cudaSetDevice(s->cfg.device);
  const int max_inflight = s->cfg.max_inflight == 1 ? 1 : 2;
  std::unique_lock<std::mutex> lk(s->mu);
  for (;;) {
    bool progress = false;
    // admission, FIFO; the allocations run without the lock
    while (!s->admit.empty()) {
      Stream& st = *s->streams[s->admit.front()];
      if (s->in_use + st.bytes > s->cfg.memory_budget) break;
      s->admit.pop_front();
      s->in_use += st.bytes;
      st.state = 4;
      const gspec_config cfg = st.cfg;
      const int id = st.id;
      Stream fresh;
      std::string aerr;
      lk.unlock();
      const bool good = admit_stream(s->cfg, cfg, id, fresh, aerr);
      lk.lock();
      take_resources(st, fresh);
      if (!good) {
        st.failed = true;
        if (s->err.empty()) s->err = aerr;
      }
      st.state = st.close_requested ? 2 : 1;
      progress = true;
      lk.unlock();
      free_stream_memory(fresh);   // whatever a failed admission left behind
      lk.lock();
    }
    bool busy = false;
    // completions of every stream, in order per stream: runs before the issue
    // pass and again after every issued block, so a long block's issue (many
    // copy pieces and launches) delays no other stream's result
    auto complete_all = [&]() {
      for (size_t kc = 0; kc < s->streams.size(); ++kc) {
        Stream& st = *s->streams[kc];
        if (st.state != 1 && st.state != 2) continue;
        while (!st.flight.empty()) {
          Flight& f = st.flight.front();
          const cudaError_t q = cudaEventQuery(f.done);
          if (q == cudaErrorNotReady) break;
          int status = GSPEC_OK;
          if (q != cudaSuccess) {
            status = GSPEC_ERR_CUDA;
            st.h->err = std::string("block failed: ") + cudaGetErrorString(q);
            st.failed = true;
          } else if (st.h->h_err && *st.h->h_err) {
            status = GSPEC_ERR_CUDA;
            st.h->err = "a bounded device wait gave up (code " + std::to_string(*st.h->h_err) + ")";
            st.failed = true;
          }
          s->results.push_back(make_result(s, st, f, status, now_s(s)));
          s->inflight_bytes -= f.bytes;
          st.flight.pop_front();
          progress = true;
          s->cv_result.notify_all();
        }
      }
    };
    complete_all();
    for (size_t k = 0; k < s->streams.size(); ++k) {
      Stream& st = *s->streams[k];
      if (st.state != 1 && st.state != 2) continue;
      // issue
      while (!st.queue.empty() && static_cast<int>(st.flight.size()) < max_inflight) {
        const Queued& q = st.queue.front();
        if (st.failed || !st.h) {
          Flight f{q.index, q.tag, q.t_submit, now_s(s), -1, nullptr, 0, -1};
          s->results.push_back(make_result(s, st, f, GSPEC_ERR_STATE, now_s(s)));
          st.queue.pop_front();
          s->cv_result.notify_all();
          progress = true;
          continue;
        }
        if (q.size > kShortBlockMax && s->cfg.inflight_bytes && s->inflight_bytes > 0 &&
            s->inflight_bytes + q.size > s->cfg.inflight_bytes)
          break;   // the GPU holds enough long blocks: wait for one to finish
        int obuf = -1;
        if ((q.index + 1) % st.info.n_blocks == 0) {
          for (size_t i = 0; i < st.hfree.size(); ++i)
            if (st.hfree[i]) {
              obuf = static_cast<int>(i);
              break;
            }
          if (obuf < 0) break;   // wait for the caller to release a result
          st.hfree[obuf] = 0;
        }
        if (!issue(s, st, q, obuf)) {
          if (obuf >= 0) st.hfree[obuf] = 1;
          continue;   // st.failed is set: the block is answered with an error above
        }
        st.queue.pop_front();
        progress = true;
        complete_all();
      }
      if (!st.flight.empty()) busy = true;
      if (st.state == 2 && stream_idle(st)) {
        if (st.h) s->launches_done += st.h->launches;
        st.state = 5;
        Stream gone;
        take_resources(gone, st);
        lk.unlock();
        free_stream_memory(gone);
        lk.lock();
        s->in_use -= st.bytes;
        st.state = 3;
        progress = true;
      }
    }
    if (s->stop) {
      bool all_idle = true;
      for (auto& up : s->streams)
        if (up->state != 3 && (!up->queue.empty() || !up->flight.empty())) all_idle = false;
      if (all_idle) break;
    }
    if (!progress) {
      // blocks on the GPU: poll their events often; otherwise sleep until work arrives
      if (busy)
        s->cv_work.wait_for(lk, std::chrono::microseconds(20));
      else
        s->cv_work.wait_for(lk, std::chrono::milliseconds(5));
    }
  }
}

Stream* find(gspec_server* s, int id) {
  if (!s || id < 0 || id >= static_cast<int>(s->streams.size())) return nullptr;
  return s->streams[id].get();
}

}  // namespace

extern "C" {

gspec_server* gspec_server_create(const gspec_server_config* cfg, char* err, size_t err_len) {
  auto report = [&](const char* m) {
    if (err && err_len) std::snprintf(err, err_len, "%s", m);
  };
  if (!cfg) {
    report("null config");
    return nullptr;
  }
  if (cfg->memory_budget == 0) {
    report("memory_budget must be > 0");
    return nullptr;
  }
  if (cudaSetDevice(cfg->device) != cudaSuccess) {
    report("cudaSetDevice failed");
    return nullptr;
  }
  auto* s = new gspec_server();
  s->cfg = *cfg;
  s->t0 = Clock::now();
  // the GPU clock against the server clock: an event on an idle stream,
  // recorded after the host time is taken
  cudaStream_t es = nullptr;
  if (cudaStreamCreateWithFlags(&es, cudaStreamNonBlocking) == cudaSuccess) {
    if (cudaEventCreate(&s->epoch) == cudaSuccess) {
      s->t_epoch = now_s(s);
      if (cudaEventRecord(s->epoch, es) != cudaSuccess || cudaEventSynchronize(s->epoch) != cudaSuccess) {
        cudaEventDestroy(s->epoch);
        s->epoch = nullptr;
      }
    }
    cudaStreamDestroy(es);
  }
  s->worker = std::thread(worker_loop, s);
  return s;
}

void gspec_server_destroy(gspec_server* s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->worker.join();
  cudaSetDevice(s->cfg.device);
  for (auto& up : s->streams) free_stream_memory(*up);
  if (s->epoch) cudaEventDestroy(s->epoch);
  delete s;
}

int gspec_stream_open(gspec_server* s, const gspec_config* cfg, int* stream_id) {
  if (!s || !cfg || !stream_id) return GSPEC_ERR_ARG;
  gspec_config c = *cfg;
  c.device = s->cfg.device;
  c.flags |= GSPEC_FLAG_NO_HOST_BUFFERS;
  gspec_info info{};
  char msg[256] = {0};
  if (gspec_query(&c, &info, msg, sizeof(msg)) != GSPEC_OK) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->err = msg;
    return GSPEC_ERR_ARG;
  }
  if (info.device_bytes > s->cfg.memory_budget) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->err = "stream needs " + std::to_string(info.device_bytes) + " device bytes, more than the budget";
    return GSPEC_ERR_ARG;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  auto st = std::make_unique<Stream>();
  st->id = static_cast<int>(s->streams.size());
  st->cfg = *cfg;
  st->info = info;
  st->bytes = info.device_bytes;
  *stream_id = st->id;
  s->admit.push_back(st->id);
  s->streams.push_back(std::move(st));
  s->cv_work.notify_all();
  return GSPEC_OK;
}

int gspec_stream_state(gspec_server* s, int stream_id) {
  if (!s) return GSPEC_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  Stream* st = find(s, stream_id);
  if (!st) return GSPEC_ERR_ARG;
  return st->state == 4 ? 0 : (st->state == 5 ? 2 : st->state);
}

int gspec_submit(gspec_server* s, int stream_id, const void* block, size_t size, uint64_t tag) {
  if (!s || !block) return GSPEC_ERR_ARG;
  const double t = now_s(s);
  std::lock_guard<std::mutex> lk(s->mu);
  Stream* st = find(s, stream_id);
  if (!st || st->state == 2 || st->state == 3 || st->state == 5 || st->close_requested) {
    s->err = "unknown or closed stream";
    return GSPEC_ERR_ARG;
  }
  if (size != st->cfg.buffer_size) {
    s->err = "Unexpected Buffer Size - Got " + std::to_string(size) + " byte, expected " +
             std::to_string(st->cfg.buffer_size) + " byte";
    return GSPEC_STOP;
  }
  st->queue.push_back({block, size, tag, st->submitted++, t});
  s->cv_work.notify_all();
  return GSPEC_OK;
}

int gspec_poll(gspec_server* s, gspec_result* results, int max, int timeout_us) {
  if (!s || !results || max <= 0) return GSPEC_ERR_ARG;
  std::unique_lock<std::mutex> lk(s->mu);
  if (s->results.empty() && timeout_us > 0)
    s->cv_result.wait_for(lk, std::chrono::microseconds(timeout_us), [&] { return !s->results.empty(); });
  int n = 0;
  while (n < max && !s->results.empty()) {
    results[n++] = s->results.front();
    s->results.pop_front();
  }
  return n;
}

int gspec_server_release(gspec_server* s, int stream_id, int buffer) {
  if (!s) return GSPEC_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  Stream* st = find(s, stream_id);
  if (!st || buffer < 0 || buffer >= static_cast<int>(st->hfree.size())) return GSPEC_ERR_ARG;
  st->hfree[buffer] = 1;
  s->cv_work.notify_all();
  return GSPEC_OK;
}

int gspec_stream_close(gspec_server* s, int stream_id) {
  if (!s) return GSPEC_ERR_ARG;
  std::lock_guard<std::mutex> lk(s->mu);
  Stream* st = find(s, stream_id);
  if (!st) return GSPEC_ERR_ARG;
  if (st->state == 0) {
    // never admitted: drop it from the admission queue
    for (auto it = s->admit.begin(); it != s->admit.end(); ++it)
      if (*it == stream_id) {
        s->admit.erase(it);
        break;
      }
    for (const Queued& q : st->queue) {
      gspec_result r{};
      r.stream = st->id;
      r.status = GSPEC_ERR_STATE;
      r.tag = q.tag;
      r.block_index = q.index;
      r.buffer = -1;
      r.t_submit = r.t_start = q.t_submit;
      r.t_done = now_s(s);
      s->results.push_back(r);
    }
    st->queue.clear();
    st->state = 3;
    s->cv_result.notify_all();
    return GSPEC_OK;
  }
  if (st->state == 4) st->close_requested = true;
  if (st->state == 1) st->state = 2;
  s->cv_work.notify_all();
  return GSPEC_OK;
}

double gspec_server_now(const gspec_server* s) { return s ? now_s(s) : 0.0; }

uint64_t gspec_server_memory_in_use(const gspec_server* s) {
  if (!s) return 0;
  std::lock_guard<std::mutex> lk(s->mu);
  return s->in_use;
}

uint64_t gspec_server_kernel_launches(const gspec_server* s) {
  if (!s) return 0;
  std::lock_guard<std::mutex> lk(s->mu);
  uint64_t n = s->launches_done;
  for (auto& up : s->streams)
    if (up->h) n += up->h->launches;
  return n;
}

const char* gspec_server_last_error(const gspec_server* s) {
  if (!s) return "null server";
  std::lock_guard<std::mutex> lk(s->mu);
  static thread_local std::string copy;
  copy = s->err;
  for (auto& up : s->streams)
    if (up->failed && up->h && !up->h->err.empty()) copy += (copy.empty() ? "" : "; ") + up->h->err;
  return copy.c_str();
}

}  // extern "C"
