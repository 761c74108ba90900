// Header-only stand-ins with the reference's own type names and signatures:
// psrdada_cpp::RawBytes (psrdada_cpp/raw_bytes.hpp:19-69) and
// psrdada_cpp::effelsberg::edd::DadaBufferLayout
// (psrdada_cpp/effelsberg/edd/DadaBufferLayout.hpp:12-54), whose constructor
// takes a ring-buffer key and reads the block size from the ring
// (edd/src/DadaBufferLayout.cpp:17-39).  Here a table of "rings" stands in
// for psrdada's shared memory.  Used to show that the drop-in template takes
// the reference's types unchanged.
#pragma once

#include <sys/types.h>

#include <cstddef>
#include <cstdint>
#include <map>

namespace psrdada_cpp {

class RawBytes {
 public:
  RawBytes(char* ptr, std::size_t total, std::size_t used = 0, bool device_memory = false)
      : _ptr(ptr), _total_bytes(total), _used_bytes(used), _on_device(device_memory) {}
  RawBytes(RawBytes const&) = delete;
  ~RawBytes() {}
  std::size_t total_bytes() const { return _total_bytes; }
  std::size_t used_bytes() const { return _used_bytes; }
  void used_bytes(std::size_t u) { _used_bytes = u; }
  char* ptr() { return _ptr; }
  bool on_device() const { return _on_device; }

 private:
  char* _ptr;
  std::size_t _total_bytes;
  std::size_t _used_bytes;
  bool _on_device;
};

// key -> data block size of the stand-in rings
inline std::map<key_t, std::size_t>& mock_rings() {
  static std::map<key_t, std::size_t> rings;
  return rings;
}

namespace effelsberg {
namespace edd {

class DadaBufferLayout {
 public:
  DadaBufferLayout() {}
  DadaBufferLayout(key_t input_key, std::size_t heapSize, std::size_t nSideChannels) {
    intitialize(input_key, heapSize, nSideChannels);
  }
  void intitialize(key_t input_key, std::size_t heapSize, std::size_t nSideChannels) {
    _input_key = input_key;
    _heapSize = heapSize;
    _nSideChannels = nSideChannels;
    _bufferSize = mock_rings()[input_key];
    const std::size_t total = heapSize + nSideChannels * sizeof(int64_t);
    _nHeaps = _bufferSize / total;
    _gapSize = _bufferSize - _nHeaps * total;
  }
  key_t getInputkey() const { return _input_key; }
  std::size_t getBufferSize() const { return _bufferSize; }
  std::size_t getHeapSize() const { return _heapSize; }
  std::size_t getNSideChannels() const { return _nSideChannels; }
  std::size_t sizeOfData() const { return _nHeaps * _heapSize; }
  std::size_t sizeOfGap() const { return _gapSize; }
  std::size_t sizeOfSideChannelData() const { return _nSideChannels * sizeof(int64_t) * _nHeaps; }
  std::size_t getNHeaps() const { return _nHeaps; }

 private:
  std::size_t _bufferSize = 0;
  key_t _input_key = 0;
  std::size_t _heapSize = 0, _nSideChannels = 0, _nHeaps = 0, _gapSize = 0;
};

}  // namespace edd
}  // namespace effelsberg
}  // namespace psrdada_cpp
