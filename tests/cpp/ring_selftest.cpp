// CPU self-test of the ring types of ring.hpp (no GPU, no page-locking): a
// producer thread writes numbered blocks of varying used size into a
// MemoryRing smaller than the stream, a DadaInputStream hands them to a
// checking handler whose DadaOutputStream copies go to a second ring, drained
// by another DadaInputStream into a SimpleFileWriter; then the file is read
// back through a FileReader.  Prints "ok <blocks>" or the first mismatch.
#include <cstdio>
#include <string>
#include <thread>

#include "psrdada_cpp_gb300/ring.hpp"

using namespace psrdada_cpp_gb300;

static char pattern(std::size_t block, std::size_t i) { return static_cast<char>((block * 131 + i * 7) & 0xff); }

struct Checker {
  DadaOutputStream<MemoryRing::Writer>& out;
  std::size_t n = 0, bad = 0, block = 0;
  void init(RawBytes& h) {
    if (std::string(h.ptr(), 6) != "HEADER") ++bad;
    out.init(h);
  }
  bool operator()(RawBytes& b) {
    if (b.used_bytes() != block - (n % 3)) ++bad;
    for (std::size_t i = 0; i < b.used_bytes(); ++i)
      if (b.ptr()[i] != pattern(n, i)) {
        ++bad;
        break;
      }
    out(b);
    ++n;
    return false;
  }
};

int main(int argc, char** argv) {
  if (argc < 2) return 2;
  const std::size_t block = 1000, nblocks = 37;
  MemoryRing in(block, 3), mid(block, 2);
  MemoryRing::Writer w(in), mw(mid);
  MemoryRing::Reader r(in), mr(mid);
  std::thread producer([&] {
    auto& hs = w.header_stream();
    auto& h = hs.next();
    std::snprintf(h.ptr(), h.total_bytes(), "HEADER test\n");
    h.used_bytes(4096);
    hs.release();
    for (std::size_t k = 0; k < nblocks; ++k) {
      auto& b = w.data_stream().next();
      const std::size_t used = block - (k % 3);
      for (std::size_t i = 0; i < used; ++i) b.ptr()[i] = pattern(k, i);
      b.used_bytes(used);
      w.data_stream().release();
    }
    w.data_stream().end_of_data();
  });
  SimpleFileWriter file(argv[1]);
  std::size_t drained = 0;
  std::thread drain([&] {
    DadaInputStream<SimpleFileWriter, MemoryRing::Reader> s(mr, file);
    drained = s.start();
  });
  DadaOutputStream<MemoryRing::Writer> os(mw);
  Checker c{os};
  c.block = block;
  DadaInputStream<Checker, MemoryRing::Reader> stream(r, c);
  const std::size_t n = stream.start();
  mw.data_stream().end_of_data();
  producer.join();
  drain.join();
  if (n != nblocks || c.bad || drained != nblocks) {
    std::printf("fail n=%zu bad=%zu drained=%zu\n", n, c.bad, drained);
    return 1;
  }
  // the file holds 4096 header bytes, then the blocks' used bytes back to back
  std::size_t total = 0;
  for (std::size_t k = 0; k < nblocks; ++k) total += block - (k % 3);
  std::FILE* f = std::fopen(argv[1], "rb");
  std::fseek(f, 0, SEEK_END);
  const long size = std::ftell(f);
  std::fclose(f);
  if (static_cast<std::size_t>(size) != 4096 + total) {
    std::printf("fail file size %ld\n", size);
    return 1;
  }
  // whole 999-byte blocks through a FileReader: every block but the last partial one
  FileReader fr(argv[1], 999);
  struct Count {
    std::size_t n = 0;
    void init(RawBytes&) {}
    bool operator()(RawBytes& b) {
      n += b.used_bytes() == 999;
      return false;
    }
  } cnt;
  DadaInputStream<Count, FileReader> fs(fr, cnt);
  const std::size_t m = fs.start();
  if (m != total / 999 || cnt.n != m) {
    std::printf("fail file blocks %zu\n", m);
    return 1;
  }
  std::printf("ok %zu\n", n);
  return 0;
}
