/*
 * gspec.h - C ABI of the GB300-native EDD gated spectrometer.
 *
 * Drop-in boundary for psrdada_cpp's GatedSpectrometer handler
 * (psrdada_cpp/effelsberg/edd/GatedSpectrometer.cuh:270-366).  Plain
 * pointers, sizes and status codes only; no C++ types or exceptions cross
 * this boundary.  The C++ template include/psrdada_cpp_gb300/GatedSpectrometer.hpp
 * and the Python module psrdada_cpp_gb300.gated_spectrometer wrap it with the
 * reference's init(RawBytes&) / operator()(RawBytes&) interface.
 *
 * Status codes: GSPEC_OK (0), GSPEC_STOP (1, the block size did not match:
 * the reference's operator() returns true), negative values are errors whose
 * text gspec_last_error() returns.
 */
#ifndef GSPEC_H
#define GSPEC_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSPEC_OK 0
#define GSPEC_STOP 1
#define GSPEC_ERR_ARG (-1)
#define GSPEC_ERR_CUDA (-2)
#define GSPEC_ERR_UNSUPPORTED (-3)
#define GSPEC_ERR_STATE (-4)

/* InputType of the reference template (edd/GatedSpectrometer.cuh:87-142). */
#define GSPEC_SINGLE_POL 0 /* SinglePolarizationInput */
#define GSPEC_DUAL_POL 1   /* DualPolarizationInput   */

/* OutputType (edd/GatedSpectrometer.cuh:207-260). */
#define GSPEC_POWER 0       /* GatedPowerSpectrumOutput */
#define GSPEC_FULL_STOKES 1 /* GatedFullStokesOutput    */

/* Gate-index convention of the side-channel items. */
#define GSPEC_INTENDED 0  /* item of the heap holding the sample; per-pol baselines */
#define GSPEC_REFERENCE 1 /* the reference's literal indexing where it stays in bounds */

/* Arithmetic form of the FFT (gspec_config.form). */
#define GSPEC_FORM_FP32 0 /* FP32 Stockham FFT on the CUDA cores */
#define GSPEC_FORM_BF16 1 /* four-step DFT-32 stages on the tensor cores, operands split into BF16 parts
                             (column pass: data 2 parts x matrix 3; row pass: 3 x 3), FP32 accumulate */
#define GSPEC_FORM_FP16 2 /* the same with FP16 hi+lo halves (3 products) */

/* Flags. */
#define GSPEC_FLAG_SATURATION_RECORD 1u /* append n_out x {sat G0, sat G1} u64 to each output */
#define GSPEC_FLAG_NO_HOST_BUFFERS 2u   /* no pinned output buffers: the handle is driven only through
                                           gspec_run_block_device, a gspec_server or a gspec_batch */
#define GSPEC_FLAG_UNGATED 4u         /* the ungated FFT spectrometer (FftSpectrometer,
                                          edd/FftSpectrometer.cuh:19-85): the block holds only
                                          samples (n_side_channels 0, heap_size ignored), every
                                          sample is transformed as it is (no gate, no baseline),
                                          single-pol power only; the handler receives n_out x
                                          nchans float32 power spectra per output block and init()
                                          appends nothing to the header */

typedef struct gspec_config {
  /* DadaBufferLayout (edd/DadaBufferLayout.hpp:20-54): the reference reads the
   * buffer size from the ring buffer (edd/src/DadaBufferLayout.cpp:17-39);
   * here the caller passes it. */
  uint64_t buffer_size;           /* bytes of one DADA data block */
  uint64_t heap_size;             /* bytes of sample data per heap */
  uint64_t n_side_channels;       /* uint64 items per heap */
  /* GatedSpectrometer constructor arguments (edd/GatedSpectrometer.cuh:292-297). */
  uint64_t selected_side_channel;
  uint64_t selected_bit;
  uint64_t fft_length;
  uint64_t naccumulate;
  uint32_t nbits;                 /* 8, 10 or 12 */
  uint32_t input_type;            /* GSPEC_SINGLE_POL / GSPEC_DUAL_POL */
  uint32_t output_type;           /* GSPEC_POWER / GSPEC_FULL_STOKES */
  uint32_t convention;            /* GSPEC_INTENDED / GSPEC_REFERENCE */
  float input_level;              /* logged only, as in the reference */
  float output_level;
  int32_t device;                 /* CUDA device ordinal */
  uint32_t flags;
  /* Schedule overrides (new in this library; 0 keeps the built-in choice).
   * The autotuner (psrdada_cpp_gb300.autotune) sets them per stream shape. */
  uint64_t tune_units;            /* shared-memory path: target work units per block (default 4 x SMs) */
  uint32_t tune_n1;               /* four-step path: first-pass length N1 (N2 = fft_length/N1 in [128, 1024]) */
  uint32_t tune_scratch_mb;       /* four-step path: scratch budget of one chunk of spectra (default 512 MiB) */
  /* CUDA priority of the handle's streams (0 default; negative = higher,
   * clamped to the device's range): a server gives latency-critical streams
   * (short blocks) precedence over long blocks of other streams. */
  int32_t stream_priority;
  /* GSPEC_FORM_FP32 (default) or a tensor-core split-precision form
   * (GSPEC_FORM_BF16 / GSPEC_FORM_FP16) for fft_length 2^16..2^20: the
   * four-step passes whose length is 1024 run as two DFT-32 GEMM stages on
   * the tensor cores (fft_length >= 2^17: N1 = 1024; 2^16: N2 = 1024). */
  uint32_t form;
} gspec_config;

typedef struct gspec_info {
  uint64_t nchans;                /* fft_length/2 + 1 */
  uint64_t n_out;                 /* output spectra per output block */
  uint64_t n_blocks;              /* input blocks integrated per output block */
  uint64_t nsamps_per_pol;        /* samples per pol per input block */
  uint64_t batch;                 /* FFT frames per pol per input block */
  uint64_t output_bytes;          /* bytes handed to the handler per output block */
  uint64_t record_bytes;          /* bytes per output spectrum record */
  uint64_t device_bytes;          /* device memory held by the handle */
  uint64_t fft_path;              /* 0 shared-memory FFT, 1 four-step FFT */
  uint64_t n1, n2;                /* four-step split (0 for the shared-memory path) */
  uint64_t kernel_launches;       /* kernels this handle has launched so far */
} gspec_info;

/* Per-kernel launch counts and device time (profiling enabled). */
typedef struct gspec_kernel_profile {
  char name[32];
  uint64_t launches;
  uint64_t timed_launches;
  double total_ms;
} gspec_kernel_profile;

/* Output of one gspec_process call: when ready != 0 the handler must be
 * called with (data, size) before the next gspec_process call. */
typedef struct gspec_output {
  char* data;
  size_t size;
  int ready;
} gspec_output;

typedef struct gspec_handle gspec_handle;

/* Replaces the GatedSpectrometer constructor
 * (edd/detail/GatedSpectrometer.cu:66-161).  Returns NULL on error and
 * writes the reason into err (if err_len > 0). */
gspec_handle* gspec_create(const gspec_config* cfg, char* err, size_t err_len);

/* Replaces GatedSpectrometer::~GatedSpectrometer (edd/detail/GatedSpectrometer.cu:164-176). */
void gspec_destroy(gspec_handle* h);

/* Replaces GatedSpectrometer::init(RawBytes&) (edd/detail/GatedSpectrometer.cu:179-215):
 * appends the spectrometer parameters to the NUL-terminated DADA header in
 * place when they fit into total_bytes.  Returns GSPEC_OK, or GSPEC_STOP
 * when the text did not fit (the reference logs a warning). */
int gspec_init(gspec_handle* h, char* header, size_t total_bytes);

/* Replaces GatedSpectrometer::operator()(RawBytes&)
 * (edd/detail/GatedSpectrometer.cu:299-365) for a block in host memory
 * (pinned or pageable).  The block is fully consumed when the call returns.
 * Returns GSPEC_STOP when used_bytes differs from the buffer size. */
int gspec_process(gspec_handle* h, const char* block, size_t used_bytes, gspec_output* out);

/* Same for a block that already resides in device memory (RawBytes with
 * on_device() == true). */
int gspec_process_device(gspec_handle* h, const void* d_block, size_t used_bytes, gspec_output* out);

/* One pass of the chain over one block in device memory, accumulated into a
 * caller-owned device output buffer (gspec_info.output_bytes without the
 * saturation record, host layout), on the caller's CUDA stream; updates the
 * baselines.  No handler pipeline, no host copies.  The caller clears d_out
 * at the start of an output block, with gspec_clear_output_device or by
 * zeroing all of it.  d_block and d_out are 16-byte aligned (GSPEC_ERR_ARG
 * otherwise). */
int gspec_run_block_device(gspec_handle* h, const void* d_block, void* d_out, void* cuda_stream);
/* Clears an output buffer of h's layout for the first block of an output
 * block, on the caller's stream (no reference counterpart: the reference
 * zeroes its accumulators with thrust::fill, edd/detail/GatedSpectrometer.cu):
 * when each block holds whole outputs (gspec_info.n_blocks == 1) every
 * spectrum value is stored by the block, so only each record's counters are
 * zeroed (nothing, where the block stores the counters too: single-pol
 * 1024-point spectra with one CTA per spectrum); otherwise the whole buffer. */
int gspec_clear_output_device(gspec_handle* h, void* d_out, void* cuda_stream);

int gspec_get_info(const gspec_handle* h, gspec_info* info);
/* Sizes of a handle for cfg without creating it (no reference counterpart):
 * fills info (kernel_launches = 0) including device_bytes, the device memory
 * gspec_create would allocate.  Needs the device to read its SM count. */
int gspec_query(const gspec_config* cfg, gspec_info* info, char* err, size_t err_len);

/* Kernel accounting (new in this library; no counterpart in the reference):
 * with profiling enabled every kernel launch is bracketed by CUDA events on
 * its stream.  gspec_get_profile synchronises the device and returns the
 * number of entries written; gspec_reset_profile clears the counters. */
int gspec_set_profiling(gspec_handle* h, int enable);
int gspec_get_profile(gspec_handle* h, gspec_kernel_profile* out, int max_entries);
int gspec_reset_profile(gspec_handle* h);
const char* gspec_last_error(const gspec_handle* h);

/* Baselines [npol][G0, G1] currently used for the next block (device copy
 * synchronised to the host) and their override (tests). */
int gspec_get_baselines(gspec_handle* h, float* out4);
int gspec_set_baselines(gspec_handle* h, const float* in4);

/* Saturation counts [n_out][G0, G1] of the last output handed out by
 * gspec_process (new in this library; no counterpart in the reference). */
int gspec_get_saturation(gspec_handle* h, uint64_t* out);

/* Page-locks (and maps) bytes of host memory at ptr for the current CUDA
 * context, so that gspec_process copies blocks from it at the host link's
 * full rate; replaces dada_cuda_dbregister, which DadaClientBase calls on
 * attach to register a ring's blocks (psrdada_cpp/src/dada_client_base.cpp:78-88).
 * gspec_unregister_host undoes it (before the memory is freed). */
int gspec_register_host(void* ptr, size_t bytes);
int gspec_unregister_host(void* ptr);

/* Synthetic DADA blocks generated on the device, the producer side of tests
 * and benchmarks; replaces the reference's dummy_data_generator
 * (psrdada_cpp/effelsberg/edd/src/dummy_data_generator.cu).
 * GSPEC_DUMMY_TWO_TONE: that program's block (8 bit only): two tones from a
 * C2R of 50 at bin nFreqs/3 and 20 at bin nFreqs/2 over the block's data
 * samples, quantised between the block's minimum and maximum to 0..255 and
 * shifted by -128 (:130-156); d_work holds 8 bytes of device memory for the
 * range.  GSPEC_DUMMY_STREAM: seeded noise (sigma) plus a tone
 * (tone_amplitude, tone_period samples per cycle) per pol, clipped to nbits,
 * packed big-endian into the heap layout (dual-pol heaps and items alternate
 * P0 P1), with the selected item of every heap carrying the diode state
 * ((global heap / diode_period_heaps) & 1) in selected_bit and, for a
 * lost_fraction of heaps, bit 63; block_index continues the stream. */
#define GSPEC_DUMMY_TWO_TONE 0u
#define GSPEC_DUMMY_STREAM 1u
typedef struct gspec_dummy_config {
  uint64_t buffer_size, heap_size, n_side_channels;
  uint32_t nbits, dual_pol;
  uint32_t mode, reserved;
  uint64_t block_index, seed;
  uint64_t selected_side_channel, selected_bit, diode_period_heaps;
  uint64_t tone_period;
  float sigma, tone_amplitude, lost_fraction, reserved2;
} gspec_dummy_config;
int gspec_dummy_block_device(const gspec_dummy_config* cfg, void* d_block, void* d_work, void* cuda_stream);
/* The same block generated on the current device and copied into host memory
 * (a convenience for producers: allocates and frees its device buffers). */
int gspec_dummy_block(const gspec_dummy_config* cfg, void* host_block);

/* VLBI: samples to 2-bit VDIF frames (replaces VLBI<Handler>,
 * psrdada_cpp/effelsberg/edd/VLBI.cuh:91-170, edd/detail/VLBI.cu): the whole
 * block is 8- or 12-bit samples; each block is quantised to 2 bits at
 * -v sigma, 0, +v sigma about its mean (pack2bit_nonLinear,
 * edd/src/VLBI.cu:183-237, with exact integer block statistics) and cut into
 * VDIF frames of the template header's data frame length; frames_per_output
 * (= 2-bit bytes per block / payload + 1) frames are handed out per call,
 * those without data marked invalid, with the reference's delay (block n at
 * call n + 3).  gspec_vlbi_init reads SYNC_TIME and SAMPLE_CLOCK_START from
 * the DADA header (edd/detail/VLBI.cu:92-134): VDIF starts at the next whole
 * second and the samples before it are dropped.  Status codes as gspec_process. */
typedef struct gspec_vlbi gspec_vlbi;
typedef struct gspec_vlbi_config {
  uint64_t buffer_size;          /* bytes per input block (all samples) */
  uint32_t nbits;                /* 8 or 12 */
  int32_t device;
  uint64_t spead_heap_size;      /* recorded only, as in the reference */
  double sample_rate;            /* samples per second */
  double digitizer_threshold;    /* v */
  uint32_t vdif_header[8];       /* template: data frame length (8-byte units, header included), station,
                                    thread, channels; epoch, second and frame number are set by init */
} gspec_vlbi_config;
typedef struct gspec_vlbi_info {
  uint64_t frame_bytes, frames_per_output, output_bytes, frames_per_second, bytes_to_skip, spill_bytes;
  uint32_t header[8];            /* the next frame's header */
  int64_t last_sum;              /* integer sum and sum of squares of the last processed block */
  uint64_t last_sum_sq;
} gspec_vlbi_info;
gspec_vlbi* gspec_vlbi_create(const gspec_vlbi_config* cfg, char* err, size_t err_len);
int gspec_vlbi_init(gspec_vlbi* h, char* header, size_t total_bytes);
int gspec_vlbi_process(gspec_vlbi* h, const char* block, size_t used_bytes, gspec_output* out);
int gspec_vlbi_get_info(gspec_vlbi* h, gspec_vlbi_info* info);
const char* gspec_vlbi_last_error(gspec_vlbi* h);
void gspec_vlbi_destroy(gspec_vlbi* h);
/* Sets a VDIF header's reference epoch (half-years since 2000) and seconds
 * since the epoch from a POSIX time (VDIFHeader::setTimeReferencesFromTimestamp,
 * edd/src/VLBI.cu:143-170); GSPEC_ERR_ARG before 2000. */
int gspec_vdif_set_time(uint32_t* header, uint64_t posix_seconds);

/* Allocation-free variant of gspec_run_block_device (no counterpart in the
 * reference).  For callers that cannot allocate device memory between blocks
 * (device memory reserved up front by a ring buffer or an outside pool,
 * real-time loops that must not pay cudaMalloc's latency): one block in
 * device memory through the chain, accumulated into the caller's d_out
 * (output layout without the saturation record), with the caller's
 * d_baselines (4 floats [pol][G0, G1], read and updated for the next block)
 * on the caller's stream (d_block and d_out 16-byte aligned, d_baselines
 * 4-byte; GSPEC_ERR_ARG otherwise).  No handle, no cudaMalloc/cudaFree: the working
 * memory is a library-owned device array of GSPEC_NOALLOC_SCRATCH_BYTES held
 * by every GPU that loads the library.  Only fft_length <= 4096; larger
 * working sets are rejected (GSPEC_ERR_UNSUPPORTED) with the reason in err.
 * cfg->device must be the current device.  The first call on a device looks
 * up the array's device address; with CUDA's default lazy module loading that
 * is also when the driver reserves the array's 32 MiB on that device, so make
 * the first call at start-up, before the caller reserves the rest of the
 * device memory for its pool and before any stream capture.  The address is
 * kept per device number: it is valid for the primary context and is not
 * looked up again after a cudaDeviceReset.  All calls share the array and it
 * keeps the last call's contents: calls that overlap on the GPU race. */
#define GSPEC_NOALLOC_SCRATCH_BYTES (32u * 1024u * 1024u)
int gspec_process_block_noalloc(const gspec_config* cfg, const void* d_block, float* d_baselines, void* d_out,
                                void* cuda_stream, char* err, size_t err_len);

/* ------------------------------------------------------------------------
 * Serving (no reference counterpart: the reference runs one
 * GatedSpectrometer per process on one ring buffer).  One server owns one
 * GPU and a scheduler thread that takes blocks from many concurrent streams
 * (each with its own fft_length, naccumulate, bit depth and pol mode), keeps
 * every admitted stream's baselines, counters and output accumulators
 * resident in device memory, and overlaps the streams' work on the device.
 * A stream is admitted when the device memory it needs (gspec_query) fits
 * into the memory budget next to the streams already admitted; until then it
 * and its blocks wait in FIFO order.  Blocks of one stream are processed in
 * submission order; each produces one result.  A result carries the output
 * block (reference layout, plus the saturation record with
 * GSPEC_FLAG_SATURATION_RECORD) when that block completed one, i.e. every
 * n_blocks blocks, with no reference pipeline delay.
 * ------------------------------------------------------------------------ */
typedef struct gspec_server gspec_server;
typedef struct gspec_server_config {
  uint64_t memory_budget;   /* bytes of device memory all admitted streams may hold */
  int32_t device;
  int32_t max_inflight;     /* blocks of one stream on the GPU at once (1 or 2; 0 = 2) */
  int32_t output_buffers;   /* pinned host output buffers per stream (0 = 2) */
  int32_t reserved;
  uint64_t inflight_bytes;  /* input bytes of all streams' long blocks (> 64 MiB) on the GPU at once
                               (0 = no limit); a long block that would exceed it waits unless no long
                               block is in flight, short blocks never wait for it.  Bounds the copy
                               and kernel queues that short blocks wait behind */
} gspec_server_config;
typedef struct gspec_result {
  int32_t stream;           /* stream id */
  int32_t status;           /* GSPEC_OK or a negative error code */
  uint64_t tag;             /* the caller's tag of the block */
  uint64_t block_index;     /* 0-based block number within the stream */
  const char* data;         /* output block, or NULL when the block completed none */
  uint64_t size;
  int32_t buffer;           /* pass to gspec_server_release once data has been consumed */
  int32_t reserved;
  double t_submit;          /* seconds on the server clock: gspec_submit called */
  double t_start;           /* the block's first copy was issued to the GPU */
  double t_done;            /* output on the host (or the block finished) */
  /* GPU-side stages of the block from CUDA events, in ms: the input copy,
   * the wait between copy and chain (earlier blocks of the stream, the
   * output accumulator), the chain's kernels, and the output copy. */
  float h2d_ms, wait_ms, chain_ms, d2h_ms;
  /* From the block's first copy issued (t_start) to the GPU starting that
   * copy, and from the GPU finishing the block to t_done, in ms (the GPU
   * clock mapped onto the server clock by an event at server creation). */
  float issue_ms, observe_ms;
} gspec_result;
gspec_server* gspec_server_create(const gspec_server_config* cfg, char* err, size_t err_len);
/* Waits for the streams' outstanding blocks, then frees everything. */
void gspec_server_destroy(gspec_server* s);
/* Opens a stream; *stream_id receives its id.  GSPEC_OK when it was
 * admitted or queued for admission, GSPEC_ERR_ARG when cfg is invalid or it
 * can never fit into the budget. */
int gspec_stream_open(gspec_server* s, const gspec_config* cfg, int* stream_id);
/* 0 waiting for admission, 1 admitted, 2 closing, 3 closed, <0 unknown id. */
int gspec_stream_state(gspec_server* s, int stream_id);
/* Queues one block.  The host memory must stay valid and unchanged until
 * the block's result has been returned by gspec_poll; page-locked memory
 * lets its copy overlap the GPU work of other blocks, and a page-locked
 * block of at most 64 MiB is read by SM loads instead of a copy engine. */
int gspec_submit(gspec_server* s, int stream_id, const void* block, size_t size, uint64_t tag);
/* Returns up to max finished results (oldest first), waiting up to
 * timeout_us microseconds for the first one. */
int gspec_poll(gspec_server* s, gspec_result* results, int max, int timeout_us);
/* Gives an output buffer back to its stream. */
int gspec_server_release(gspec_server* s, int stream_id, int buffer);
/* Closes a stream once its queued blocks are done and frees its memory,
 * which may admit waiting streams. */
int gspec_stream_close(gspec_server* s, int stream_id);
double gspec_server_now(const gspec_server* s);
uint64_t gspec_server_memory_in_use(const gspec_server* s);
/* Kernels launched by all streams so far. */
uint64_t gspec_server_kernel_launches(const gspec_server* s);
const char* gspec_server_last_error(const gspec_server* s);

/* ------------------------------------------------------------------------
 * Batch of uneven streams in one CUDA graph (no reference counterpart).
 * Each member stream has its own configuration and device input block;
 * gspec_batch_run launches one graph in which every stream's chain runs in
 * its own branch, so the streams' kernels share the GPU.  Member i's output
 * accumulator is complete after the steps where (step + 1) % n_blocks_i == 0.
 * ------------------------------------------------------------------------ */
typedef struct gspec_batch gspec_batch;
gspec_batch* gspec_batch_create(const gspec_config* cfgs, int n, char* err, size_t err_len);
void gspec_batch_destroy(gspec_batch* b);
int gspec_batch_size(const gspec_batch* b);
int gspec_batch_get_info(const gspec_batch* b, int i, gspec_info* info);
/* Device input block of member i (buffer_size bytes) read by the next run.
 * Every member has two input buffers and runs alternate between them: the
 * blocks of step k + 1 can be copied in while step k runs, ordered after
 * step k - 1 (the last run that read the same buffer). */
void* gspec_batch_input(gspec_batch* b, int i);
/* Copies one block (host or device memory, buffer_size bytes) into member
 * i's input on the caller's stream. */
int gspec_batch_set_input(gspec_batch* b, int i, const void* src, size_t bytes, void* cuda_stream);
/* Copies member i's output accumulator (output layout without the
 * saturation record) to dst (host or device memory) on the caller's stream
 * and waits for the copy. */
int gspec_batch_read_output(gspec_batch* b, int i, void* dst, size_t bytes, void* cuda_stream);
/* The same copy enqueued on the caller's stream without waiting. */
int gspec_batch_copy_output(gspec_batch* b, int i, void* dst, size_t bytes, void* cuda_stream);
/* Device output accumulator of member i (output layout without the
 * saturation record) and whether the last run completed it. */
int gspec_batch_output(gspec_batch* b, int i, void** d_out, uint64_t* bytes, int* complete);
/* One step: one block through every member, as one graph launch on the
 * caller's stream (captured at the first call). */
int gspec_batch_run(gspec_batch* b, void* cuda_stream);
/* Kernel nodes in one step's graph and steps run so far. */
uint64_t gspec_batch_kernels_per_step(const gspec_batch* b);
uint64_t gspec_batch_steps(const gspec_batch* b);
const char* gspec_batch_last_error(const gspec_batch* b);

/* Test entry points of single stages on device memory. */
/* Tensor-core DFT-1024 (form GSPEC_FORM_BF16 or GSPEC_FORM_FP16) of
 * ntransforms (a multiple of 4) contiguous FP32 complex sequences: the
 * split-precision stage of the four-step form on its own (no reference
 * counterpart: the reference calls cuFFT). */
int gspec_tc_dft1024_device(const void* d_in, void* d_out, uint32_t ntransforms, int form, void* cuda_stream);
/* Unpacker::unpack<nbits> (edd/src/Unpacker.cu:124-140): contiguous packed
 * big-endian samples -> float. */
int gspec_unpack_device(const void* d_raw, uint32_t nbits, uint64_t nsamples, float* d_out, void* cuda_stream);
/* gating (edd/src/GatedSpectrometer.cu:22-90) of a whole block with the
 * handle's current baselines; d_gated is [npol][G0, G1][nsamps_per_pol]
 * float.  Does not change the handle's state. */
int gspec_gate_device(gspec_handle* h, const void* d_block, float* d_gated, void* cuda_stream);

#ifdef __cplusplus
}
#endif

#endif /* GSPEC_H */
