// extern "C" exports of the reference's host-side reference code, compiled
// together with the reference's own source files (see build_ref.sh):
//   * UnpackerTester::unpacker_{8,10,12}_to_32_c_reference
//     (psrdada_cpp/effelsberg/edd/test/src/UnpackerTester.cu:41-201)
//   * DetectorAccumulatorTester::detect_c_reference
//     (psrdada_cpp/effelsberg/edd/test/src/DetectorAccumulatorTester.cu:33-62)
//   * stokes_IQUV (psrdada_cpp/effelsberg/edd/src/GatedSpectrometer.cu:125-131)
#include <cstdint>
#include <cstring>
#include "psrdada_cpp/effelsberg/edd/test/UnpackerTester.cuh"
#include "psrdada_cpp/effelsberg/edd/test/DetectorAccumulatorTester.cuh"
#include "psrdada_cpp/effelsberg/edd/GatedSpectrometer.cuh"

namespace edd = psrdada_cpp::effelsberg::edd;

struct UnpackAccess : public edd::test::UnpackerTester {
  using edd::test::UnpackerTester::unpacker_8_to_32_c_reference;
  using edd::test::UnpackerTester::unpacker_10_to_32_c_reference;
  using edd::test::UnpackerTester::unpacker_12_to_32_c_reference;
};

struct DetectAccess : public edd::test::DetectorAccumulatorTester {
  using edd::test::DetectorAccumulatorTester::detect_c_reference;
};

extern "C" {

// words: big-endian packed uint64 words as stored in memory; returns the
// number of samples written to out.
size_t ref_unpack(const uint64_t* words, size_t nwords, int nbits, float* out) {
  UnpackAccess t;
  edd::test::UnpackerTester::InputType in(words, words + nwords);
  edd::test::UnpackerTester::OutputType o;
  if (nbits == 8) t.unpacker_8_to_32_c_reference(in, o);
  else if (nbits == 10) t.unpacker_10_to_32_c_reference(in, o);
  else if (nbits == 12) t.unpacker_12_to_32_c_reference(in, o);
  else return 0;
  std::memcpy(out, o.data(), o.size() * sizeof(float));
  return o.size();
}

size_t ref_detect_int8(const float* in_xy, size_t n, int nchans, int tscrunch, float scale, float offset,
                       int8_t* out) {
  DetectAccess t;
  edd::test::DetectorAccumulatorTester::InputType in(n);
  for (size_t i = 0; i < n; ++i) in[i] = make_float2(in_xy[2 * i], in_xy[2 * i + 1]);
  edd::test::DetectorAccumulatorTester::OutputType o;
  t.detect_c_reference(in, o, nchans, tscrunch, scale, offset);
  std::memcpy(out, o.data(), o.size());
  return o.size();
}

void ref_stokes_iquv(float p1x, float p1y, float p2x, float p2y, float* iquv) {
  float I, Q, U, V;
  edd::stokes_IQUV(make_float2(p1x, p1y), make_float2(p2x, p2y), I, Q, U, V);
  iquv[0] = I; iquv[1] = Q; iquv[2] = U; iquv[3] = V;
}

}  // extern "C"
