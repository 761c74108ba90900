// Ring-buffer sources and sinks around the gated spectrometer: the step
// before the path (a DADA ring's header and data blocks, page-locked so the
// block's host-to-device copy runs at the host link's rate) and the step
// after it (an output ring or a file).
//
// Each type restates a psrdada_cpp interface with the same semantics:
//  * MemoryRing: an in-process ring of data blocks plus a header block with
//    psrdada's reader/writer protocol.  The reader's header_stream() /
//    data_stream() give next() / release() / at_end() as
//    DadaReadClient::HeaderStream / DataStream
//    (psrdada_cpp/src/dada_read_client.cpp:73-190).  The writer's streams give
//    next() / release() as DadaWriteClient's (psrdada_cpp/dada_write_client.hpp);
//    the writer marks the end of data (ipcbuf_enable_eod).  With page_lock the
//    ring's memory is registered with CUDA, as dada_cuda_dbregister does for a
//    psrdada ring (psrdada_cpp/src/dada_client_base.cpp:78-88).
//  * FileReader: the same reader interface over a DADA file (a header block,
//    then whole data blocks), as FileInputStream reads one
//    (psrdada_cpp/detail/file_input_stream.cpp:29-66).
//  * DadaInputStream<Handler, Reader>: the handler loop of
//    psrdada_cpp/detail/dada_input_stream.cpp:21-52 (init with the header
//    block, then operator() with each data block until the handler asks to
//    stop or the data ends) over one reader.
//  * DadaOutputStream<Writer>: a handler that copies the header and every
//    block it is given into a ring (psrdada_cpp/src/dada_output_stream.cpp:19-35).
//  * SimpleFileWriter and NullSink: psrdada_cpp/src/simple_file_writer.cpp:25-42
//    and psrdada_cpp/dada_null_sink.hpp.
//  * With HAVE_PSRDADA, PsrdadaReadClient / PsrdadaWriteClient give the same
//    interface over a real psrdada ring (dada_hdu), written against psrdada's
//    public C API.
//
// Error convention: std::runtime_error, as the reference's clients.
#pragma once

#include <condition_variable>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../gspec.h"
#include "raw_bytes.hpp"

#ifdef HAVE_PSRDADA
extern "C" {
#include "dada_cuda.h"
#include "dada_hdu.h"
#include "ipcbuf.h"
#include "ipcio.h"
}
#endif

namespace psrdada_cpp_gb300 {

// ------------------------------------------------------------- MemoryRing
class MemoryRing {
 public:
  // nbufs data blocks of data_block_bytes and one header block; page_lock
  // registers the whole ring with CUDA (gspec_register_host) so that copies
  // from its blocks to the device run at the host link's full rate.
  MemoryRing(std::size_t data_block_bytes, std::size_t nbufs, std::size_t header_bytes = 4096,
             bool page_lock = false)
      : _block(data_block_bytes), _nbufs(nbufs), _header_bytes(header_bytes), _used(nbufs, 0) {
    if (nbufs == 0 || data_block_bytes == 0) throw std::runtime_error("MemoryRing: empty ring");
    // 4096-byte aligned blocks (page-lockable, 16-byte aligned for the device kernels)
    _stride = (data_block_bytes + 4095) / 4096 * 4096;
    _hstride = (header_bytes + 4095) / 4096 * 4096;
    _bytes = _hstride + _stride * nbufs;
    _base = static_cast<char*>(std::aligned_alloc(4096, _bytes));
    if (!_base) throw std::runtime_error("MemoryRing: out of host memory");
    std::memset(_base, 0, _bytes);
    if (page_lock) {
      if (gspec_register_host(_base, _bytes) != GSPEC_OK) {
        std::free(_base);
        throw std::runtime_error("MemoryRing: page-locking the ring failed");
      }
      _locked = true;
    }
  }
  ~MemoryRing() {
    if (_locked) gspec_unregister_host(_base);
    std::free(_base);
  }
  MemoryRing(const MemoryRing&) = delete;
  MemoryRing& operator=(const MemoryRing&) = delete;

  std::size_t data_buffer_size() const { return _block; }
  std::size_t header_buffer_size() const { return _header_bytes; }
  std::size_t nbufs() const { return _nbufs; }
  bool page_locked() const { return _locked; }

  // --- the writer's streams
  class HeaderWriteStream {
   public:
    explicit HeaderWriteStream(MemoryRing& r) : _r(r) {}
    RawBytes& next() {
      std::unique_lock<std::mutex> lk(_r._m);
      if (_cur) throw std::runtime_error("Previous header block not released");
      _r._cv.wait(lk, [&] { return !_r._header_full; });
      _cur.reset(new RawBytes(_r._base, _r._header_bytes, 0));
      return *_cur;
    }
    void release() {
      std::lock_guard<std::mutex> lk(_r._m);
      if (!_cur) throw std::runtime_error("No header block to be released");
      _r._header_used = _cur->used_bytes();
      _r._header_full = true;
      _cur.reset();
      _r._cv.notify_all();
    }

   private:
    MemoryRing& _r;
    std::unique_ptr<RawBytes> _cur;
  };
  class DataWriteStream {
   public:
    explicit DataWriteStream(MemoryRing& r) : _r(r) {}
    // the next free block (waits while the ring is full)
    RawBytes& next() {
      std::unique_lock<std::mutex> lk(_r._m);
      if (_cur) throw std::runtime_error("Previous data block not released");
      if (_r._eod) throw std::runtime_error("Data block requested after the end of data");
      _r._cv.wait(lk, [&] { return _r._nfull < _r._nbufs; });
      _cur.reset(new RawBytes(_r.block_ptr(_r._wpos), _r._block, 0));
      return *_cur;
    }
    // marks the block full with its used_bytes
    void release() {
      std::lock_guard<std::mutex> lk(_r._m);
      if (!_cur) throw std::runtime_error("No data block to be released");
      _r._used[_r._wpos] = _cur->used_bytes();
      _r._wpos = (_r._wpos + 1) % _r._nbufs;
      ++_r._nfull;
      ++_r._written;
      _cur.reset();
      _r._cv.notify_all();
    }
    // no more data after the blocks released so far (ipcbuf_enable_eod)
    void end_of_data() {
      std::lock_guard<std::mutex> lk(_r._m);
      _r._eod = true;
      _r._cv.notify_all();
    }

   private:
    MemoryRing& _r;
    std::unique_ptr<RawBytes> _cur;
  };

  // --- the reader's streams
  class HeaderReadStream {
   public:
    explicit HeaderReadStream(MemoryRing& r) : _r(r) {}
    RawBytes& next() {
      std::unique_lock<std::mutex> lk(_r._m);
      if (_cur) throw std::runtime_error("Previous header block not released");
      _r._cv.wait(lk, [&] { return _r._header_full; });
      _cur.reset(new RawBytes(_r._base, _r._header_bytes, _r._header_used));
      return *_cur;
    }
    void release() {
      std::lock_guard<std::mutex> lk(_r._m);
      if (!_cur) throw std::runtime_error("No header block to be released");
      _r._header_full = false;
      _cur.reset();
      _r._cv.notify_all();
    }
    bool at_end() const { return false; }

   private:
    MemoryRing& _r;
    std::unique_ptr<RawBytes> _cur;
  };
  class DataReadStream {
   public:
    explicit DataReadStream(MemoryRing& r) : _r(r) {}
    // the oldest full block (waits while the ring is empty); throws at the
    // end of data, as DadaReadClient::DataStream::next does when no block opens
    RawBytes& next() {
      std::unique_lock<std::mutex> lk(_r._m);
      if (_cur) throw std::runtime_error("Previous data block not released");
      _r._cv.wait(lk, [&] { return _r._nfull > 0 || _r._eod; });
      if (_r._nfull == 0) throw std::runtime_error("Could not open block to read: end of data");
      _cur.reset(new RawBytes(_r.block_ptr(_r._rpos), _r._block, _r._used[_r._rpos]));
      return *_cur;
    }
    void release() {
      std::lock_guard<std::mutex> lk(_r._m);
      if (!_cur) throw std::runtime_error("No data block to be released");
      _r._rpos = (_r._rpos + 1) % _r._nbufs;
      --_r._nfull;
      _cur.reset();
      _r._cv.notify_all();
    }
    // every block written before the end-of-data mark has been read; waits
    // while the writer has neither written more nor marked the end
    bool at_end() const {
      std::unique_lock<std::mutex> lk(_r._m);
      _r._cv.wait(lk, [&] { return _r._nfull > 0 || _r._eod; });
      return _r._eod && _r._nfull == 0;
    }

   private:
    MemoryRing& _r;
    std::unique_ptr<RawBytes> _cur;
  };

  // the two sides of the ring
  class Writer {
   public:
    explicit Writer(MemoryRing& r) : _h(r), _d(r) {}
    HeaderWriteStream& header_stream() { return _h; }
    DataWriteStream& data_stream() { return _d; }

   private:
    HeaderWriteStream _h;
    DataWriteStream _d;
  };
  class Reader {
   public:
    explicit Reader(MemoryRing& r) : _r(r), _h(r), _d(r) {}
    HeaderReadStream& header_stream() { return _h; }
    DataReadStream& data_stream() { return _d; }
    std::size_t data_buffer_size() const { return _r.data_buffer_size(); }
    std::size_t header_buffer_size() const { return _r.header_buffer_size(); }

   private:
    MemoryRing& _r;
    HeaderReadStream _h;
    DataReadStream _d;
  };

  std::size_t blocks_written() const {
    std::lock_guard<std::mutex> lk(_m);
    return _written;
  }

 private:
  char* block_ptr(std::size_t i) { return _base + _hstride + i * _stride; }

  std::size_t _block, _nbufs, _header_bytes, _stride = 0, _hstride = 0, _bytes = 0;
  char* _base = nullptr;
  bool _locked = false;
  mutable std::mutex _m;
  mutable std::condition_variable _cv;
  std::vector<std::size_t> _used;
  std::size_t _wpos = 0, _rpos = 0, _nfull = 0, _written = 0, _header_used = 0;
  bool _eod = false, _header_full = false;
};

// ------------------------------------------------------------- FileReader
// A DADA file (header_bytes of header, then data blocks of block_bytes) with
// the reader interface.  Blocks are read into one buffer (page-locked when
// page_lock is set) that is valid until release().
class FileReader {
 public:
  FileReader(const std::string& path, std::size_t block_bytes, std::size_t header_bytes = 4096,
             bool page_lock = false)
      : _in(path, std::ios::binary), _block(block_bytes), _hbytes(header_bytes), _h(*this), _d(*this) {
    if (!_in.is_open()) throw std::runtime_error("Could not open file " + path);
    _in.seekg(0, std::ios::end);
    _size = static_cast<std::size_t>(_in.tellg());
    _in.seekg(0, std::ios::beg);
    _hbuf.assign(header_bytes, 0);
    _buf = static_cast<char*>(std::aligned_alloc(4096, (block_bytes + 4095) / 4096 * 4096));
    if (!_buf) throw std::runtime_error("FileReader: out of host memory");
    if (page_lock) {
      if (gspec_register_host(_buf, (block_bytes + 4095) / 4096 * 4096) != GSPEC_OK) {
        std::free(_buf);
        throw std::runtime_error("FileReader: page-locking the block buffer failed");
      }
      _locked = true;
    }
  }
  ~FileReader() {
    if (_locked) gspec_unregister_host(_buf);
    std::free(_buf);
  }
  FileReader(const FileReader&) = delete;

  class HeaderStream {
   public:
    explicit HeaderStream(FileReader& f) : _f(f) {}
    RawBytes& next() {
      if (_cur) throw std::runtime_error("Previous header block not released");
      _f._in.seekg(0);
      _f._in.read(_f._hbuf.data(), static_cast<std::streamsize>(_f._hbytes));
      if (!_f._in) throw std::runtime_error("Could not get header");
      _cur.reset(new RawBytes(_f._hbuf.data(), _f._hbytes, _f._hbytes));
      return *_cur;
    }
    void release() {
      if (!_cur) throw std::runtime_error("No header block to be released");
      _cur.reset();
    }
    bool at_end() const { return false; }

   private:
    FileReader& _f;
    std::unique_ptr<RawBytes> _cur;
  };
  class DataStream {
   public:
    explicit DataStream(FileReader& f) : _f(f) {}
    RawBytes& next() {
      if (_cur) throw std::runtime_error("Previous data block not released");
      if (at_end()) throw std::runtime_error("Could not open block to read: end of data");
      _f._in.seekg(static_cast<std::streamoff>(_f._hbytes + _idx * _f._block));
      _f._in.read(_f._buf, static_cast<std::streamsize>(_f._block));
      if (!_f._in) throw std::runtime_error("Could not read data block");
      _cur.reset(new RawBytes(_f._buf, _f._block, _f._block));
      return *_cur;
    }
    void release() {
      if (!_cur) throw std::runtime_error("No data block to be released");
      _cur.reset();
      ++_idx;
    }
    // no whole block left in the file
    bool at_end() const { return _f._hbytes + (_idx + 1) * _f._block > _f._size; }

   private:
    FileReader& _f;
    std::unique_ptr<RawBytes> _cur;
    std::size_t _idx = 0;
  };
  HeaderStream& header_stream() { return _h; }
  DataStream& data_stream() { return _d; }
  std::size_t data_buffer_size() const { return _block; }
  std::size_t header_buffer_size() const { return _hbytes; }

 private:
  std::ifstream _in;
  std::size_t _block, _hbytes, _size = 0;
  std::vector<char> _hbuf;
  char* _buf = nullptr;
  bool _locked = false;
  HeaderStream _h;
  DataStream _d;
};

// -------------------------------------------------------- DadaInputStream
// detail/dada_input_stream.cpp:21-52 over one reader: the header block to
// handler.init, then every data block to handler() until it returns true
// (stop) or the reader reaches the end of data.  The reference re-attaches a
// new read client after each end of data; here the caller starts the stream
// again with a new reader.
template <class HandlerType, class ReaderType>
class DadaInputStream {
 public:
  DadaInputStream(ReaderType& reader, HandlerType& handler) : _reader(reader), _handler(handler) {}
  // returns the number of data blocks handed to the handler
  std::size_t start() {
    if (_running) throw std::runtime_error("Stream is already running");
    _running = true;
    std::size_t n = 0;
    auto& hs = _reader.header_stream();
    _handler.init(hs.next());
    hs.release();
    auto& ds = _reader.data_stream();
    bool handler_stop = false;
    while (!_stop && !handler_stop) {
      handler_stop = _handler(ds.next());
      ds.release();
      ++n;
      if (ds.at_end()) break;
    }
    _running = false;
    return n;
  }
  void stop() { _stop = true; }

 private:
  ReaderType& _reader;
  HandlerType& _handler;
  bool _stop = false, _running = false;
};

// ------------------------------------------------------- DadaOutputStream
// src/dada_output_stream.cpp:19-35: the header and every block the handler
// gets are copied into the writer's next header / data block.
template <class WriterType>
class DadaOutputStream {
 public:
  explicit DadaOutputStream(WriterType& writer) : _writer(writer) {}
  void init(RawBytes& in) {
    auto& stream = _writer.header_stream();
    auto& buffer = stream.next();
    if (in.used_bytes() > buffer.total_bytes()) throw std::runtime_error("header larger than the header block");
    std::memcpy(buffer.ptr(), in.ptr(), in.used_bytes());
    buffer.used_bytes(in.used_bytes());
    stream.release();
  }
  bool operator()(RawBytes& in) {
    auto& stream = _writer.data_stream();
    auto& out = stream.next();
    if (in.used_bytes() > out.total_bytes()) throw std::runtime_error("output larger than the ring's blocks");
    std::memcpy(out.ptr(), in.ptr(), in.used_bytes());
    out.used_bytes(in.used_bytes());
    stream.release();
    return false;
  }
  WriterType const& client() const { return _writer; }

 private:
  WriterType& _writer;
};

// ------------------------------------------------------ SimpleFileWriter
// src/simple_file_writer.cpp:25-42: 4096 bytes of header, then every block.
class SimpleFileWriter {
 public:
  explicit SimpleFileWriter(const std::string& filename) : _out(filename, std::ios::out | std::ios::binary) {
    if (!_out.is_open()) throw std::runtime_error("Could not open file " + filename);
  }
  void init(RawBytes& block) { _out.write(block.ptr(), 4096); }
  void init(RawBytes& block, std::size_t size) { _out.write(block.ptr(), static_cast<std::streamsize>(size)); }
  bool operator()(RawBytes& block) {
    _out.write(block.ptr(), static_cast<std::streamsize>(block.used_bytes()));
    _out.flush();
    block.used_bytes(block.total_bytes());
    return false;
  }

 private:
  std::ofstream _out;
};

// psrdada_cpp/dada_null_sink.hpp
class NullSink {
 public:
  void init(RawBytes&) {}
  bool operator()(RawBytes&) { return false; }
};

#ifdef HAVE_PSRDADA
// ------------------------------------------------- psrdada ring clients
// The reader and writer interfaces over a psrdada ring buffer (dada_hdu), as
// DadaReadClient / DadaWriteClient (psrdada_cpp/src/dada_read_client.cpp,
// psrdada_cpp/src/dada_write_client.cpp), with the ring's blocks registered
// with CUDA on attach (dada_cuda_dbregister, src/dada_client_base.cpp:78-88).
class PsrdadaClientBase {
 protected:
  PsrdadaClientBase(key_t key, bool cuda_register) {
    _hdu = dada_hdu_create(nullptr);
    dada_hdu_set_key(_hdu, key);
    if (dada_hdu_connect(_hdu) < 0) throw std::runtime_error("Unable to connect to hdu with key " + std::to_string(key));
    if (cuda_register) dada_cuda_dbregister(_hdu);
  }
  ~PsrdadaClientBase() {
    dada_hdu_disconnect(_hdu);
    dada_hdu_destroy(_hdu);
  }
  dada_hdu_t* _hdu = nullptr;

 public:
  std::size_t data_buffer_size() const { return ipcbuf_get_bufsz(reinterpret_cast<ipcbuf_t*>(_hdu->data_block)); }
  std::size_t header_buffer_size() const { return ipcbuf_get_bufsz(_hdu->header_block); }
};

class PsrdadaReadClient : public PsrdadaClientBase {
 public:
  explicit PsrdadaReadClient(key_t key, bool cuda_register = true)
      : PsrdadaClientBase(key, cuda_register), _h(*this), _d(*this) {
    if (dada_hdu_lock_read(_hdu) < 0) throw std::runtime_error("Error locking HDU with key: " + std::to_string(key));
  }
  ~PsrdadaReadClient() { dada_hdu_unlock_read(_hdu); }

  class HeaderStream {
   public:
    explicit HeaderStream(PsrdadaReadClient& c) : _c(c) {}
    RawBytes& next() {
      if (_cur) throw std::runtime_error("Previous header block not released");
      uint64_t nbytes = 0;
      char* p = ipcbuf_get_next_read(_c._hdu->header_block, &nbytes);
      if (!p) throw std::runtime_error("Could not get header");
      _cur.reset(new RawBytes(p, _c.header_buffer_size(), nbytes));
      return *_cur;
    }
    void release() {
      if (!_cur) throw std::runtime_error("No header block to be released");
      if (ipcbuf_mark_cleared(_c._hdu->header_block) < 0) throw std::runtime_error("Could not mark cleared header block");
      _cur.reset();
    }
    bool at_end() const { return ipcbuf_eod(_c._hdu->header_block); }

   private:
    PsrdadaReadClient& _c;
    std::unique_ptr<RawBytes> _cur;
  };
  class DataStream {
   public:
    explicit DataStream(PsrdadaReadClient& c) : _c(c) {}
    RawBytes& next() {
      if (_cur) throw std::runtime_error("Previous data block not released");
      uint64_t nbytes = 0, idx = 0;
      char* p = ipcio_open_block_read(_c._hdu->data_block, &nbytes, &idx);
      if (!p) throw std::runtime_error("Could not open block to read");
      _cur.reset(new RawBytes(p, _c.data_buffer_size(), nbytes));
      return *_cur;
    }
    void release() {
      if (!_cur) throw std::runtime_error("No data block to be released");
      if (ipcio_close_block_read(_c._hdu->data_block, _cur->used_bytes()) < 0)
        throw std::runtime_error("Could not close ipcio data block");
      _cur.reset();
    }
    bool at_end() const { return ipcbuf_eod(reinterpret_cast<ipcbuf_t*>(_c._hdu->data_block)); }

   private:
    PsrdadaReadClient& _c;
    std::unique_ptr<RawBytes> _cur;
  };
  HeaderStream& header_stream() { return _h; }
  DataStream& data_stream() { return _d; }

 private:
  HeaderStream _h;
  DataStream _d;
};

class PsrdadaWriteClient : public PsrdadaClientBase {
 public:
  explicit PsrdadaWriteClient(key_t key, bool cuda_register = false)
      : PsrdadaClientBase(key, cuda_register), _h(*this), _d(*this) {
    if (dada_hdu_lock_write(_hdu) < 0) throw std::runtime_error("Error locking HDU with key: " + std::to_string(key));
  }
  ~PsrdadaWriteClient() { dada_hdu_unlock_write(_hdu); }

  class HeaderStream {
   public:
    explicit HeaderStream(PsrdadaWriteClient& c) : _c(c) {}
    RawBytes& next() {
      if (_cur) throw std::runtime_error("Previous header block not released");
      char* p = ipcbuf_get_next_write(_c._hdu->header_block);
      if (!p) throw std::runtime_error("Could not get next header block");
      _cur.reset(new RawBytes(p, _c.header_buffer_size(), 0));
      return *_cur;
    }
    void release() {
      if (!_cur) throw std::runtime_error("No header block to be released");
      if (ipcbuf_mark_filled(_c._hdu->header_block, _cur->used_bytes()) < 0)
        throw std::runtime_error("Could not mark filled header block");
      _cur.reset();
    }

   private:
    PsrdadaWriteClient& _c;
    std::unique_ptr<RawBytes> _cur;
  };
  class DataStream {
   public:
    explicit DataStream(PsrdadaWriteClient& c) : _c(c) {}
    RawBytes& next() {
      if (_cur) throw std::runtime_error("Previous data block not released");
      uint64_t idx = 0;
      char* p = ipcio_open_block_write(_c._hdu->data_block, &idx);
      if (!p) throw std::runtime_error("Could not open block to write");
      _cur.reset(new RawBytes(p, _c.data_buffer_size(), 0));
      return *_cur;
    }
    void release() {
      if (!_cur) throw std::runtime_error("No data block to be released");
      if (ipcio_close_block_write(_c._hdu->data_block, _cur->used_bytes()) < 0)
        throw std::runtime_error("Could not close ipcio data block");
      _cur.reset();
    }

   private:
    PsrdadaWriteClient& _c;
    std::unique_ptr<RawBytes> _cur;
  };
  HeaderStream& header_stream() { return _h; }
  DataStream& data_stream() { return _d; }

 private:
  HeaderStream _h;
  DataStream _d;
};
#endif  // HAVE_PSRDADA

}  // namespace psrdada_cpp_gb300
