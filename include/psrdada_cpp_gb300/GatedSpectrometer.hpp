// C++ drop-in for psrdada_cpp's EDD gated spectrometer handler.
//
// GatedSpectrometer<HandlerType, InputType, OutputType> keeps the reference's
// constructor arguments and its init(RawBytes&) / operator()(RawBytes&) pair
// (psrdada_cpp/effelsberg/edd/GatedSpectrometer.cuh:270-366), so a
// DadaInputStream<GatedSpectrometer<...>> or FileInputStream drives it
// unchanged.  The work runs in libgspec.so through the C ABI of gspec.h; no
// exception crosses that boundary, errors are rethrown here as
// std::runtime_error like the reference's CUDA_ERROR_CHECK
// (psrdada_cpp/cuda_utils.hpp:25-47).
//
// The RawBytes type is a template parameter: psrdada_cpp::RawBytes
// (psrdada_cpp/raw_bytes.hpp:19-69) works as is; psrdada_cpp_gb300::RawBytes
// below is a stand-alone equivalent for builds without psrdada_cpp.
#pragma once

#include <cstddef>
#include <cstdint>
#include <stdexcept>
#include <string>

#include "../gspec.h"
#include "raw_bytes.hpp"

namespace psrdada_cpp_gb300 {

// DadaBufferLayout (psrdada_cpp/effelsberg/edd/DadaBufferLayout.hpp:20-54).
// The reference reads the buffer size from the ring buffer
// (edd/src/DadaBufferLayout.cpp:17-39); here it is passed in, e.g. from
// DadaReadClient::data_buffer_size().
class DadaBufferLayout {
 public:
  DadaBufferLayout() = default;
  DadaBufferLayout(std::size_t buffer_size, std::size_t heap_size, std::size_t n_side_channels) {
    intitialize(buffer_size, heap_size, n_side_channels);
  }
  // spelled as in the reference
  void intitialize(std::size_t buffer_size, std::size_t heap_size, std::size_t n_side_channels) {
    _buffer_size = buffer_size;
    _heap_size = heap_size;
    _nsc = n_side_channels;
    const std::size_t total = heap_size + n_side_channels * sizeof(int64_t);
    _n_heaps = total ? buffer_size / total : 0;
    _gap = buffer_size - _n_heaps * total;
  }
  std::size_t getBufferSize() const { return _buffer_size; }
  std::size_t getHeapSize() const { return _heap_size; }
  std::size_t getNSideChannels() const { return _nsc; }
  std::size_t sizeOfData() const { return _n_heaps * _heap_size; }
  std::size_t sizeOfGap() const { return _gap; }
  std::size_t sizeOfSideChannelData() const { return _nsc * sizeof(int64_t) * _n_heaps; }
  std::size_t getNHeaps() const { return _n_heaps; }

 private:
  std::size_t _buffer_size = 0, _heap_size = 0, _nsc = 0, _n_heaps = 0, _gap = 0;
};

// Template tags of the reference's instantiations
// (edd/src/GatedSpectrometer_cli.cu:105-126).
struct SinglePolarizationInput {
  static constexpr uint32_t value = GSPEC_SINGLE_POL;
};
struct DualPolarizationInput {
  static constexpr uint32_t value = GSPEC_DUAL_POL;
};
struct GatedPowerSpectrumOutput {
  static constexpr uint32_t value = GSPEC_POWER;
};
struct GatedFullStokesOutput {
  static constexpr uint32_t value = GSPEC_FULL_STOKES;
};

template <class HandlerType, class InputType, class OutputType, class RawBytesType = RawBytes>
class GatedSpectrometer {
 public:
  // edd/GatedSpectrometer.cuh:292-297.  The layout is any type with the
  // getters of psrdada_cpp::effelsberg::edd::DadaBufferLayout
  // (edd/DadaBufferLayout.hpp:31-51: getBufferSize, getHeapSize,
  // getNSideChannels), so the reference's own layout, constructed from a ring
  // buffer key, passes unchanged; DadaBufferLayout above is the stand-alone
  // equivalent.
  template <class LayoutType>
  GatedSpectrometer(const LayoutType& bufferLayout, std::size_t selectedSideChannel, std::size_t selectedBit,
                    std::size_t fft_length, std::size_t naccumulate, std::size_t nbits, float input_level,
                    float output_level, HandlerType& handler, uint32_t convention = GSPEC_INTENDED,
                    int device = 0, uint32_t flags = 0)
      : _handler(handler) {
    gspec_config c{};
    c.buffer_size = bufferLayout.getBufferSize();
    c.heap_size = bufferLayout.getHeapSize();
    c.n_side_channels = bufferLayout.getNSideChannels();
    c.selected_side_channel = selectedSideChannel;
    c.selected_bit = selectedBit;
    c.fft_length = fft_length;
    c.naccumulate = naccumulate;
    c.nbits = static_cast<uint32_t>(nbits);
    c.input_type = InputType::value;
    c.output_type = OutputType::value;
    c.convention = convention;
    c.input_level = input_level;
    c.output_level = output_level;
    c.device = device;
    c.flags = flags;
    char err[512] = {0};
    _h = gspec_create(&c, err, sizeof(err));
    if (!_h) throw std::runtime_error(std::string("GatedSpectrometer: ") + err);
  }
  ~GatedSpectrometer() { gspec_destroy(_h); }
  GatedSpectrometer(const GatedSpectrometer&) = delete;
  GatedSpectrometer& operator=(const GatedSpectrometer&) = delete;

  // edd/detail/GatedSpectrometer.cu:179-215: append the parameters to the
  // header (a warning, not an error, when they do not fit), then forward.
  void init(RawBytesType& block) {
    const int rc = gspec_init(_h, block.ptr(), block.total_bytes());
    if (rc < 0) throw std::runtime_error(gspec_last_error(_h));
    _handler.init(block);
  }

  // edd/detail/GatedSpectrometer.cu:299-365: returns true to stop the stream.
  bool operator()(RawBytesType& block) {
    gspec_output out{};
    const int rc = block.on_device() ? gspec_process_device(_h, block.ptr(), block.used_bytes(), &out)
                                     : gspec_process(_h, block.ptr(), block.used_bytes(), &out);
    if (rc == GSPEC_STOP) return true;
    if (rc < 0) throw std::runtime_error(gspec_last_error(_h));
    if (out.ready) {
      // valid only during the handler call, as in the reference
      RawBytesType bytes(out.data, out.size, out.size);
      _handler(bytes);
    }
    return false;
  }

  gspec_info info() const {
    gspec_info i{};
    gspec_get_info(_h, &i);
    return i;
  }
  gspec_handle* handle() { return _h; }

 private:
  HandlerType& _handler;
  gspec_handle* _h = nullptr;
};

}  // namespace psrdada_cpp_gb300
