// C++ drop-in for psrdada_cpp's ungated EDD FFT spectrometer handler.
//
// FftSpectrometer<HandlerType> keeps the reference's constructor arguments
// (buffer_bytes, fft_length, naccumulate, nbits, input_level, output_level,
// handler) and its init(RawBytes&) / operator()(RawBytes&) pair
// (psrdada_cpp/effelsberg/edd/FftSpectrometer.cuh:19-85).  It runs the gated
// spectrometer's kernels with GSPEC_FLAG_UNGATED (include/gspec.h): every
// fft_length samples of the block are one R2C frame, naccumulate frames add
// up to one float32 power spectrum of fft_length/2 + 1 channels, and the
// handler receives the block's spectra three calls later, as in the
// reference.  The reference's in-place R2C stride overlap, never-zeroed
// power buffers and frame-count rounding (edd/detail/FftSpectrometer.cu:
// 54-56,103-107,133-147) are not reproduced: each output block holds exactly
// its input block's frames.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "../gspec.h"
#include "raw_bytes.hpp"

namespace psrdada_cpp_gb300 {

template <class HandlerType, class RawBytesType = RawBytes>
class FftSpectrometer {
 public:
  // edd/FftSpectrometer.cuh:29-36
  FftSpectrometer(std::size_t buffer_bytes, std::size_t fft_length, std::size_t naccumulate, std::size_t nbits,
                  float input_level, float output_level, HandlerType& handler, int device = 0)
      : _handler(handler) {
    gspec_config c{};
    c.buffer_size = buffer_bytes;
    c.heap_size = buffer_bytes;
    c.n_side_channels = 0;
    c.fft_length = fft_length;
    c.naccumulate = naccumulate;
    c.nbits = static_cast<uint32_t>(nbits);
    c.input_type = GSPEC_SINGLE_POL;
    c.output_type = GSPEC_POWER;
    c.convention = GSPEC_INTENDED;
    c.input_level = input_level;
    c.output_level = output_level;
    c.device = device;
    c.flags = GSPEC_FLAG_UNGATED;
    char err[512] = {0};
    _h = gspec_create(&c, err, sizeof(err));
    if (!_h) throw std::runtime_error(std::string("FftSpectrometer: ") + err);
  }
  ~FftSpectrometer() { gspec_destroy(_h); }
  FftSpectrometer(const FftSpectrometer&) = delete;
  FftSpectrometer& operator=(const FftSpectrometer&) = delete;

  // edd/detail/FftSpectrometer.cu:119-123: the header goes to the handler unchanged
  void init(RawBytesType& block) { _handler.init(block); }

  // edd/detail/FftSpectrometer.cu:149-183: returns true to stop the stream
  bool operator()(RawBytesType& block) {
    gspec_output out{};
    const int rc = block.on_device() ? gspec_process_device(_h, block.ptr(), block.used_bytes(), &out)
                                     : gspec_process(_h, block.ptr(), block.used_bytes(), &out);
    if (rc == GSPEC_STOP) return true;
    if (rc < 0) throw std::runtime_error(gspec_last_error(_h));
    if (out.ready) {
      RawBytesType bytes(out.data, out.size, out.size);
      return _handler(bytes);
    }
    return false;
  }

  gspec_info info() const {
    gspec_info i{};
    gspec_get_info(_h, &i);
    return i;
  }

 private:
  HandlerType& _handler;
  gspec_handle* _h = nullptr;
};

}  // namespace psrdada_cpp_gb300
