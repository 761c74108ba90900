// The gated spectrometer between two rings, as a psrdada deployment wires it
// (a DadaReadClient feeding DadaInputStream<GatedSpectrometer<DadaOutputStream>>,
// edd/src/GatedSpectrometer_cli.cu:45-126): a producer thread copies a DADA
// file into a page-locked input MemoryRing, the spectrometer's output blocks
// go through a DadaOutputStream into an output ring, and a drain thread
// writes that ring to a file with SimpleFileWriter.
//
//   ring_pipeline <in.dada> <out.dat> <block_bytes> <heap> <nsc> <fft> <nacc> <nbits> <dual> <out_bytes>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <thread>

#include "psrdada_cpp_gb300/GatedSpectrometer.hpp"
#include "psrdada_cpp_gb300/ring.hpp"

using namespace psrdada_cpp_gb300;

template <class Spec>
std::size_t run(Spec& spec, MemoryRing::Reader& reader) {
  DadaInputStream<Spec, MemoryRing::Reader> stream(reader, spec);
  return stream.start();
}

int main(int argc, char** argv) {
  if (argc < 11) {
    std::cerr << "usage: " << argv[0] << " in out block_bytes heap nsc fft nacc nbits dual out_bytes\n";
    return 2;
  }
  const std::size_t block = std::strtoull(argv[3], nullptr, 10);
  const std::size_t fft = std::strtoull(argv[6], nullptr, 10), nacc = std::strtoull(argv[7], nullptr, 10);
  const std::size_t nbits = std::strtoull(argv[8], nullptr, 10), out_bytes = std::strtoull(argv[10], nullptr, 10);
  const bool dual = std::atoi(argv[9]) != 0;
  DadaBufferLayout layout(block, std::strtoull(argv[4], nullptr, 10), std::strtoull(argv[5], nullptr, 10));
  try {
    MemoryRing in(block, 4, 4096, /*page_lock=*/true), out(out_bytes, 3, 4096);
    MemoryRing::Writer in_w(in), out_w(out);
    MemoryRing::Reader in_r(in), out_r(out);
    std::thread producer([&] {
      FileReader file(argv[1], block);
      auto& fh = file.header_stream().next();
      auto& h = in_w.header_stream().next();
      std::copy(fh.ptr(), fh.ptr() + fh.used_bytes(), h.ptr());
      h.used_bytes(fh.used_bytes());
      in_w.header_stream().release();
      file.header_stream().release();
      while (!file.data_stream().at_end()) {
        auto& src = file.data_stream().next();
        auto& dst = in_w.data_stream().next();
        std::copy(src.ptr(), src.ptr() + src.used_bytes(), dst.ptr());
        dst.used_bytes(src.used_bytes());
        in_w.data_stream().release();
        file.data_stream().release();
      }
      in_w.data_stream().end_of_data();
    });
    SimpleFileWriter writer(argv[2]);
    std::size_t drained = 0;
    std::thread drain([&] {
      DadaInputStream<SimpleFileWriter, MemoryRing::Reader> s(out_r, writer);
      drained = s.start();
    });
    DadaOutputStream<MemoryRing::Writer> sink(out_w);
    std::size_t n;
    if (dual) {
      GatedSpectrometer<DadaOutputStream<MemoryRing::Writer>, DualPolarizationInput, GatedFullStokesOutput> spec(
          layout, 0, 0, fft, nacc, nbits, 100.f, 100.f, sink);
      n = run(spec, in_r);
    } else {
      GatedSpectrometer<DadaOutputStream<MemoryRing::Writer>, SinglePolarizationInput, GatedPowerSpectrumOutput>
          spec(layout, 0, 0, fft, nacc, nbits, 100.f, 100.f, sink);
      n = run(spec, in_r);
    }
    out_w.data_stream().end_of_data();
    producer.join();
    drain.join();
    std::printf("blocks %zu outputs %zu page_locked %d\n", n, drained, in.page_locked() ? 1 : 0);
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
