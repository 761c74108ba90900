// Non-owning view of a buffer with a total and a used size, as
// psrdada_cpp::RawBytes (psrdada_cpp/raw_bytes.hpp:19-69): the type every
// handler's init() and operator() take.
#pragma once

#include <cstddef>

namespace psrdada_cpp_gb300 {

class RawBytes {
 public:
  RawBytes(char* ptr, std::size_t total, std::size_t used = 0, bool device_memory = false)
      : _ptr(ptr), _total(total), _used(used), _on_device(device_memory) {}
  RawBytes(const RawBytes&) = delete;
  std::size_t total_bytes() const { return _total; }
  std::size_t used_bytes() const { return _used; }
  void used_bytes(std::size_t u) { _used = u; }
  char* ptr() { return _ptr; }
  bool on_device() const { return _on_device; }

 private:
  char* _ptr;
  std::size_t _total;
  std::size_t _used;
  bool _on_device;
};

}  // namespace psrdada_cpp_gb300
