/*
 * CPU restatement of the EDD gated-spectrometer chain in C with OpenMP.
 *
 * TEST AND CPU-BASELINE INFRASTRUCTURE ONLY: used by tests/ as a second checker and
 * by bench.py as the timed CPU path ("cpu_baseline", "--impl reference").
 * The product path never links it.
 *
 * It follows the same steps as oracle/gspec_oracle.py:
 *   unpack   edd/test/src/UnpackerTester.cu:41-201 (big-endian bit stream)
 *   layout   edd/src/DadaBufferLayout.cpp:17-39, de-interleave
 *            edd/src/GatedSpectrometer.cu:212-230,261-306
 *   gate     edd/src/GatedSpectrometer.cu:22-59 ((v - b) * m + b in float)
 *   baseline edd/src/GatedSpectrometer.cu:98-118 (exact integer sums)
 *   R2C      the reference uses cuFFT; FFTW is not available here, so a
 *            radix-2 FP32 complex FFT written for this file computes two real
 *            transforms per complex one (z = a + i b)
 *   detect   edd/DetectorAccumulator.cuh:40-61, Stokes
 *            edd/src/GatedSpectrometer.cu:125-169
 * Output spectra are accumulated into the reference's output layout
 * (edd/src/GatedSpectrometer.cu:346-384,430-527).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

typedef struct {
  uint64_t buffer_size, heap_size, nsc, sel, bitpos, fft_length, naccumulate;
  uint32_t nbits, dual, convention;
  /* derived */
  uint64_t n_heaps, gap, data_bytes, sc_off, nsamps, items_per_pol, n_blocks, batch, nacc, n_out, C, rec;
} cpu_cfg;

int cpu_configure(cpu_cfg* c) {
  uint64_t scs = c->nsc * 8;
  c->n_heaps = c->buffer_size / (c->heap_size + scs);
  if (!c->n_heaps) return -1;
  c->gap = c->buffer_size - c->n_heaps * (c->heap_size + scs);
  c->data_bytes = c->n_heaps * c->heap_size;
  c->sc_off = c->data_bytes + c->gap;
  uint64_t pol_bytes = c->dual ? c->data_bytes / 2 : c->data_bytes;
  c->nsamps = pol_bytes * 8 / c->nbits;
  c->items_per_pol = c->dual ? c->n_heaps * c->nsc / 2 : c->n_heaps * c->nsc;
  uint64_t N = c->fft_length, per_out = N * c->naccumulate;
  if (per_out <= c->nsamps) {
    if (c->nsamps % per_out) return -2;
    c->n_blocks = 1;
  } else {
    if (per_out % c->nsamps) return -3;
    c->n_blocks = per_out / c->nsamps;
  }
  c->batch = c->nsamps / N;
  c->nacc = c->naccumulate / c->n_blocks;
  c->n_out = c->batch / c->nacc;
  c->C = N / 2 + 1;
  c->rec = (c->dual ? 8 : 2) * (c->C * 4 + 8);
  return 0;
}

static inline const uint8_t* pol_base(const cpu_cfg* c, const uint8_t* block, int pol, uint64_t byte) {
  if (!c->dual) return block + byte;
  uint64_t h = byte / c->heap_size;
  return block + (2 * h + pol) * c->heap_size + (byte - h * c->heap_size);
}

static inline uint64_t item_index(const cpu_cfg* c, uint64_t s) {
  if (c->convention == 1) {
    uint64_t L = c->nsamps / c->n_out, step = c->items_per_pol / c->n_out;
    uint64_t j = s / L, t = s - j * L;
    return j * step + (t / c->heap_size) * c->nsc + c->sel;
  }
  return ((s * c->nbits) / (8 * c->heap_size)) * c->nsc + c->sel;
}

static inline uint64_t load_item(const cpu_cfg* c, const uint8_t* block, uint64_t idx) {
  const uint64_t* items = (const uint64_t*)(block + c->sc_off);
  if (!c->dual) return items[idx];
  uint64_t a = items[2 * idx], b = items[2 * idx + 1];
  if (c->convention == 1) return (a != 0 || b != 0) ? 1u : 0u;
  return a | b;
}

/* ---------------------------------------------------------------- FFT */
typedef struct { float x, y; } cpx;

static void fft_tables(uint32_t N, cpx* tw, uint32_t* rev) {
  int L = 0;
  while ((1u << L) < N) ++L;
  for (uint32_t i = 0; i < N / 2; ++i) {
    double a = -2.0 * M_PI * (double)i / (double)N;
    tw[i].x = (float)cos(a);
    tw[i].y = (float)sin(a);
  }
  for (uint32_t i = 0; i < N; ++i) {
    uint32_t r = 0;
    for (int b = 0; b < L; ++b) r |= ((i >> b) & 1u) << (L - 1 - b);
    rev[i] = r;
  }
}

/* in-place iterative radix-2 DIT, input in bit-reversed order */
static void fft_run(cpx* a, uint32_t N, const cpx* tw) {
  for (uint32_t len = 2; len <= N; len <<= 1) {
    uint32_t half = len >> 1, stride = N / len;
    for (uint32_t i = 0; i < N; i += len) {
      for (uint32_t j = 0; j < half; ++j) {
        cpx w = tw[j * stride];
        cpx u = a[i + j], v = a[i + j + half];
        cpx t = {v.x * w.x - v.y * w.y, v.x * w.y + v.y * w.x};
        a[i + j].x = u.x + t.x;
        a[i + j].y = u.y + t.y;
        a[i + j + half].x = u.x - t.x;
        a[i + j + half].y = u.y - t.y;
      }
    }
  }
}

/* ---------------------------------------------------------------- block */
/* Process one block into out (host output layout, accumulating) and sat
 * ([n_out][2]); baselines [npol][2] are read and updated; pol_stats receives
 * the per-pol counts and sums of this block.  Returns 0 on success. */
int cpu_run_block(const cpu_cfg* c, const uint8_t* block, uint8_t* out, uint64_t* sat, float* baselines,
                  int nthreads) {
  const uint32_t N = (uint32_t)c->fft_length;
  const int npol = c->dual ? 2 : 1;
  const uint64_t C = c->C;
  const int vals = c->dual ? 8 : 2;
  cpx* tw = (cpx*)malloc(sizeof(cpx) * (N / 2 + 1));
  uint32_t* rev = (uint32_t*)malloc(sizeof(uint32_t) * N);
  if (!tw || !rev) return -1;
  fft_tables(N, tw, rev);
  const float b[4] = {baselines[0], baselines[1], baselines[2], baselines[3]};
  long long sums[2][2] = {{0, 0}, {0, 0}};
  unsigned long long cnts[2][2] = {{0, 0}, {0, 0}};
  const int lo = -(1 << (c->nbits - 1)), hi = (1 << (c->nbits - 1)) - 1;
  int nt = 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
  nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#endif
  /* per-thread partial spectra of the current output, summed in thread order */
  float* partial = (float*)malloc(sizeof(float) * (size_t)nt * vals * C);
  if (!partial) return -1;
#pragma omp parallel num_threads(nt)
  {
    int tid = 0;
#ifdef _OPENMP
    tid = omp_get_thread_num();
#endif
    cpx* z = (cpx*)malloc(sizeof(cpx) * N * 2);
    float* acc = partial + (size_t)tid * vals * C;
    long long ls[2][2] = {{0, 0}, {0, 0}};
    unsigned long long lc[2][2] = {{0, 0}, {0, 0}};
    for (long long k = 0; k < (long long)c->n_out; ++k) {
      memset(acc, 0, sizeof(float) * vals * C);
      unsigned long long n0 = 0, n1 = 0, s0c = 0, s1c = 0;
#pragma omp for schedule(static)
      for (long long fr = 0; fr < (long long)c->nacc; ++fr) {
        uint64_t f = (uint64_t)k * c->nacc + fr;
        for (uint32_t n = 0; n < N; ++n) {
          uint64_t s = f * N + n;
          uint64_t it = load_item(c, block, item_index(c, s));
          int bit = (int)((it >> c->bitpos) & 1u), lost = (int)(it >> 63);
          int m0 = !bit && !lost, m1 = bit && !lost;
          float g[2][2];
          for (int p = 0; p < npol; ++p) {
            uint64_t sb = s * c->nbits;
            const uint8_t* q = pol_base(c, block, p, sb >> 3);
            int32_t v = c->nbits == 8 ? (int32_t)(int8_t)q[0] : 0;
            if (c->nbits != 8) {
              uint32_t sh = (uint32_t)(sb & 7);
              uint32_t w = ((uint32_t)q[0] << 16) | ((uint32_t)q[1] << 8) | (uint32_t)q[2];
              uint32_t u = (w >> (24 - sh - c->nbits)) & ((1u << c->nbits) - 1u);
              v = (int32_t)(u ^ (1u << (c->nbits - 1))) - (int32_t)(1u << (c->nbits - 1));
            }
            float vf = (float)v;
            const float d0 = vf - b[2 * p], d1 = vf - b[2 * p + 1];
            g[p][0] = m0 ? d0 + b[2 * p] : b[2 * p];
            g[p][1] = m1 ? d1 + b[2 * p + 1] : b[2 * p + 1];
            lc[p][0] += m0;
            lc[p][1] += m1;
            ls[p][0] += m0 ? v : 0;
            ls[p][1] += m1 ? v : 0;
            n0 += m0;
            n1 += m1;
            int satv = (v == lo) || (v == hi);
            s0c += m0 && satv;
            s1c += m1 && satv;
          }
          uint32_t r = rev[n];
          if (!c->dual) {
            z[r].x = g[0][0];
            z[r].y = g[0][1];
          } else {
            z[r].x = g[0][0];
            z[r].y = g[1][0];
            z[N + r].x = g[0][1];
            z[N + r].y = g[1][1];
          }
        }
        fft_run(z, N, tw);
        if (c->dual) fft_run(z + N, N, tw);
        for (uint64_t ch = 0; ch < C; ++ch) {
          uint64_t cm = (N - ch) & (N - 1);
          if (!c->dual) {
            cpx a = z[ch], bb = z[cm];
            float sx = a.x + bb.x, sy = a.y - bb.y, dx = a.x - bb.x, dy = a.y + bb.y;
            acc[ch] += 0.25f * (sx * sx + sy * sy);
            acc[C + ch] += 0.25f * (dx * dx + dy * dy);
          } else {
            for (int gt = 0; gt < 2; ++gt) {
              cpx a = z[gt * N + ch], bb = z[gt * N + cm];
              float p1x = 0.5f * (a.x + bb.x), p1y = 0.5f * (a.y - bb.y);
              float p2x = 0.5f * (a.y + bb.y), p2y = -0.5f * (a.x - bb.x);
              float a1 = p1x * p1x + p1y * p1y, a2 = p2x * p2x + p2y * p2y;
              acc[(0 + gt) * C + ch] += a1 + a2;
              acc[(2 + gt) * C + ch] += a1 - a2;
              acc[(4 + gt) * C + ch] += 2.f * (p1x * p2x + p1y * p2y);
              acc[(6 + gt) * C + ch] += -2.f * (p1y * p2x - p1x * p2y);
            }
          }
        }
      }
      /* the implicit barrier of the frame loop has passed: sum the threads'
       * partials in a fixed order */
      float* of = (float*)(out + (uint64_t)k * c->rec);
#pragma omp for schedule(static)
      for (long long i = 0; i < (long long)vals * (long long)C; ++i) {
        float v = 0.f;
        for (int t = 0; t < nt; ++t) v += partial[(size_t)t * vals * C + i];
        of[i] += v;
      }
      uint64_t* cnt = (uint64_t*)(out + (uint64_t)k * c->rec + (uint64_t)vals * C * 4);
#pragma omp atomic
      cnt[0] += n0;
#pragma omp atomic
      cnt[1] += n1;
#pragma omp atomic
      sat[2 * k] += s0c;
#pragma omp atomic
      sat[2 * k + 1] += s1c;
#pragma omp barrier
      if (c->dual && tid == 0)
        for (int rr = 1; rr < 4; ++rr) {
          cnt[2 * rr] = cnt[0];
          cnt[2 * rr + 1] = cnt[1];
        }
    }
#pragma omp critical
    {
      for (int p = 0; p < 2; ++p)
        for (int q = 0; q < 2; ++q) {
          sums[p][q] += ls[p][q];
          cnts[p][q] += lc[p][q];
        }
    }
    free(z);
  }
  free(partial);
  /* baselines for the next block */
  unsigned long long tot[2] = {0, 0};
  for (uint64_t k = 0; k < c->n_out; ++k) {
    const uint64_t* cnt = (const uint64_t*)(out + k * c->rec + (uint64_t)vals * C * 4);
    tot[0] += cnt[0];
    tot[1] += cnt[1];
  }
  for (int p = 0; p < npol; ++p) {
    for (int q = 0; q < 2; ++q) {
      unsigned long long den = cnts[p][q];
      if (c->convention == 1) {
        den = tot[q];
        if (npol == 2 && p == 0) den -= cnts[1][q];
      }
      baselines[2 * p + q] = den ? (float)((double)sums[p][q] / (double)den) : 0.f;
    }
  }
  free(tw);
  free(rev);
  return 0;
}

int cpu_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
