// C++ drop-in for psrdada_cpp's VLBI handler (8/12-bit EDD samples to 2-bit
// VDIF frames): VDIFHeaderView / VDIFHeader with the reference's accessors
// (psrdada_cpp/effelsberg/edd/VLBI.cuh:20-84; field layout of the VDIF
// specification 1.1.1) and VLBI<HandlerType> with the reference's
// constructor, init(RawBytes&) and operator()(RawBytes&)
// (edd/VLBI.cuh:91-170) over gspec_vlbi_* of gspec.h.  Differences from the
// reference: exact integer block statistics; a frame's validity bit
// describes that frame (the reference copies each header before updating
// the bit, so it marks validity one frame late); setRealDataType clears the
// data-type bit of word 3 (the reference clears bit 31 of word 0).
#pragma once

#include <cstddef>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>

#include "../gspec.h"
#include "raw_bytes.hpp"

namespace psrdada_cpp_gb300 {

constexpr std::size_t vlbiHeaderSize = 8 * 32 / 8;   // bytes: 8 words of 32 bit

class VDIFHeaderView {
 public:
  explicit VDIFHeaderView(const uint32_t* data) : data(data) {}
  void setDataLocation(const uint32_t* d) { data = d; }
  const uint32_t* getDataLocation() const { return data; }
  uint32_t getVersionNumber() const { return bits(2, 29, 31); }
  bool isValid() const { return bits(0, 31, 31) == 0; }
  uint32_t getSecondsFromReferenceEpoch() const { return bits(0, 0, 29); }
  uint32_t getReferenceEpoch() const { return bits(1, 24, 29); }
  uint32_t getDataFrameNumber() const { return bits(1, 0, 23); }
  uint32_t getDataFrameLength() const { return bits(2, 0, 23); }
  uint32_t getNumberOfChannels() const { return bits(2, 24, 28); }
  bool isRealDataType() const { return bits(3, 31, 31) == 0; }
  bool isComplexDataType() const { return bits(3, 31, 31) == 1; }
  uint32_t getBitsPerSample() const { return bits(3, 26, 30); }
  uint32_t getThreadId() const { return bits(3, 16, 25); }
  uint32_t getStationId() const { return bits(3, 0, 15); }

 protected:
  uint32_t bits(int w, int first, int last) const {
    const uint32_t mask = last - first == 31 ? 0xFFFFFFFFu : ((1u << (last - first + 1)) - 1u);
    return (data[w] >> first) & mask;
  }
  const uint32_t* data;
};

class VDIFHeader : public VDIFHeaderView {
 public:
  VDIFHeader() : VDIFHeaderView(_words) {
    std::memset(_words, 0, sizeof(_words));
    set(2, 29, 31, 1);   // version 1
  }
  VDIFHeader(const VDIFHeader& v) : VDIFHeaderView(_words) { std::memcpy(_words, v.getDataLocation(), sizeof(_words)); }
  VDIFHeader& operator=(const VDIFHeader& o) {
    std::memcpy(_words, o.getDataLocation(), sizeof(_words));
    return *this;
  }
  uint32_t* getData() { return _words; }
  void setInvalid() { set(0, 31, 31, 1); }
  void setValid() { set(0, 31, 31, 0); }
  void setSecondsFromReferenceEpoch(uint32_t v) { set(0, 0, 29, v); }
  void setReferenceEpoch(uint32_t v) { set(1, 24, 29, v); }
  void setTimeReferencesFromTimestamp(std::size_t t) {
    if (gspec_vdif_set_time(_words, t) != GSPEC_OK) throw std::runtime_error("Cannot encode time before 1 Jan 2000");
  }
  void setDataFrameNumber(uint32_t v) { set(1, 0, 23, v); }
  void setDataFrameLength(uint32_t v) { set(2, 0, 23, v); }
  void setNumberOfChannels(uint32_t v) { set(2, 24, 28, v); }
  void setComplexDataType() { set(3, 31, 31, 1); }
  void setRealDataType() { set(3, 31, 31, 0); }
  void setBitsPerSample(uint32_t v) { set(3, 26, 30, v); }
  void setThreadId(uint32_t v) { set(3, 16, 25, v); }
  void setStationId(uint32_t v) { set(3, 0, 15, v); }

 private:
  void set(int w, int first, int last, uint32_t v) {
    const uint32_t width = static_cast<uint32_t>(last - first + 1);
    if (width < 32 && v >= (1u << width)) throw std::runtime_error("Value does not fit into bitrange");
    const uint32_t mask = width == 32 ? 0xFFFFFFFFu : (((1u << width) - 1u) << first);
    _words[w] = (_words[w] & ~mask) | ((v << first) & mask);
  }
  uint32_t _words[8];
};

template <class HandlerType, class RawBytesType = RawBytes>
class VLBI {
 public:
  // edd/VLBI.cuh:106-110
  VLBI(std::size_t buffer_bytes, std::size_t input_bitDepth, std::size_t speadHeapSize, double sampleRate,
       double digitizer_threshold, const VDIFHeader& vdifHeader, HandlerType& handler, int device = 0)
      : _handler(handler) {
    gspec_vlbi_config c{};
    c.buffer_size = buffer_bytes;
    c.nbits = static_cast<uint32_t>(input_bitDepth);
    c.device = device;
    c.spead_heap_size = speadHeapSize;
    c.sample_rate = sampleRate;
    c.digitizer_threshold = digitizer_threshold;
    std::memcpy(c.vdif_header, vdifHeader.getDataLocation(), sizeof(c.vdif_header));
    char err[512] = {0};
    _h = gspec_vlbi_create(&c, err, sizeof(err));
    if (!_h) throw std::runtime_error(std::string("VLBI: ") + err);
  }
  ~VLBI() { gspec_vlbi_destroy(_h); }
  VLBI(const VLBI&) = delete;
  VLBI& operator=(const VLBI&) = delete;

  // edd/detail/VLBI.cu:92-134: without SYNC_TIME / SAMPLE_CLOCK_START the
  // reference logs a warning and returns without calling the handler
  void init(RawBytesType& block) {
    const int rc = gspec_vlbi_init(_h, block.ptr(), block.total_bytes());
    if (rc < 0) throw std::runtime_error(gspec_vlbi_last_error(_h));
    if (rc == GSPEC_STOP) return;
    _handler.init(block);
  }

  // edd/detail/VLBI.cu:137-354
  bool operator()(RawBytesType& block) {
    gspec_output out{};
    const int rc = gspec_vlbi_process(_h, block.ptr(), block.used_bytes(), &out);
    if (rc == GSPEC_STOP) return true;
    if (rc < 0) throw std::runtime_error(gspec_vlbi_last_error(_h));
    if (out.ready) {
      RawBytesType bytes(out.data, out.size, out.size);
      _handler(bytes);
    }
    return false;
  }

  gspec_vlbi_info info() const {
    gspec_vlbi_info i{};
    gspec_vlbi_get_info(_h, &i);
    return i;
  }

 private:
  HandlerType& _handler;
  gspec_vlbi* _h = nullptr;
};

}  // namespace psrdada_cpp_gb300
