// A DADA-file pipeline written against the drop-in C++ template, the way
// psrdada_cpp's gated-spectrometer CLI wires FileInputStream ->
// GatedSpectrometer -> SimpleFileWriter (edd/src/GatedSpectrometer_cli.cu:45-126,
// psrdada_cpp/detail/file_input_stream.cpp:29-66, src/simple_file_writer.cpp:25-42).
//
//   compile_handler <in.dada> <out.dat> <block_bytes> <heap> <nsc> <fft> <nacc> <nbits> <dual>
//
// Reads a 4096-byte header and then whole blocks, writes the 4096-byte header
// (with the spectrometer parameters appended) and every output block.
//
// Built with -DUSE_REFERENCE_TYPES the program uses the reference's own type
// names and signatures instead of the stand-alone ones: psrdada_cpp::RawBytes
// and psrdada_cpp::effelsberg::edd::DadaBufferLayout constructed from a ring
// key, as edd/src/GatedSpectrometer_cli.cu:45-102 does (header-only
// stand-ins in reference_types_mock.hpp).
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <iostream>
#include <vector>

#include "psrdada_cpp_gb300/GatedSpectrometer.hpp"

#ifdef USE_REFERENCE_TYPES
#include "reference_types_mock.hpp"
using psrdada_cpp::RawBytes;
#else
using psrdada_cpp_gb300::RawBytes;
#endif

struct FileSink {
  std::ofstream out;
  explicit FileSink(const char* path) : out(path, std::ios::binary) {}
  void init(RawBytes& block) { out.write(block.ptr(), 4096); }
  bool operator()(RawBytes& block) {
    out.write(block.ptr(), static_cast<std::streamsize>(block.used_bytes()));
    return false;
  }
};

template <class Handler>
std::size_t file_input_stream(const char* path, std::size_t block_bytes, Handler& handler) {
  std::ifstream in(path, std::ios::binary);
  std::vector<char> header(4096, 0), data(block_bytes);
  in.read(header.data(), 4096);
  RawBytes hb(header.data(), 4096, 4096);
  handler.init(hb);
  std::size_t n = 0;
  while (in.read(data.data(), static_cast<std::streamsize>(block_bytes))) {
    RawBytes db(data.data(), block_bytes, block_bytes);
    ++n;
    if (handler(db)) break;
  }
  return n;
}

int main(int argc, char** argv) {
  if (argc < 10) {
    std::cerr << "usage: " << argv[0] << " in out block_bytes heap nsc fft nacc nbits dual\n";
    return 2;
  }
  const std::size_t block = std::strtoull(argv[3], nullptr, 10);
#ifdef USE_REFERENCE_TYPES
  const key_t input_key = 0xdada;
  psrdada_cpp::mock_rings()[input_key] = block;
  psrdada_cpp::effelsberg::edd::DadaBufferLayout layout(input_key, std::strtoull(argv[4], nullptr, 10),
                                                         std::strtoull(argv[5], nullptr, 10));
#else
  psrdada_cpp_gb300::DadaBufferLayout layout(block, std::strtoull(argv[4], nullptr, 10),
                                              std::strtoull(argv[5], nullptr, 10));
#endif
  const std::size_t fft = std::strtoull(argv[6], nullptr, 10), nacc = std::strtoull(argv[7], nullptr, 10);
  const std::size_t nbits = std::strtoull(argv[8], nullptr, 10);
  FileSink sink(argv[2]);
  try {
    std::size_t n;
    if (std::atoi(argv[9])) {
      psrdada_cpp_gb300::GatedSpectrometer<FileSink, psrdada_cpp_gb300::DualPolarizationInput,
                                           psrdada_cpp_gb300::GatedFullStokesOutput, RawBytes>
          spec(layout, 0, 0, fft, nacc, nbits, 100.f, 100.f, sink);
      n = file_input_stream(argv[1], block, spec);
    } else {
      psrdada_cpp_gb300::GatedSpectrometer<FileSink, psrdada_cpp_gb300::SinglePolarizationInput,
                                           psrdada_cpp_gb300::GatedPowerSpectrumOutput, RawBytes>
          spec(layout, 0, 0, fft, nacc, nbits, 100.f, 100.f, sink);
      n = file_input_stream(argv[1], block, spec);
    }
    std::printf("blocks %zu\n", n);
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
