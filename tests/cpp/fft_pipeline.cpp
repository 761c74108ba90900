// The ungated FFT spectrometer in the reference's CLI wiring
// (edd/src/fft_spectrometer_cli.cu: DadaInputStream -> FftSpectrometer ->
// SimpleFileWriter), reading a DADA file through FileReader.
//
//   fft_pipeline <in.dada> <out.dat> <block_bytes> <fft> <nacc> <nbits>
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "psrdada_cpp_gb300/FftSpectrometer.hpp"
#include "psrdada_cpp_gb300/ring.hpp"

using namespace psrdada_cpp_gb300;

int main(int argc, char** argv) {
  if (argc < 7) {
    std::cerr << "usage: " << argv[0] << " in out block_bytes fft nacc nbits\n";
    return 2;
  }
  const std::size_t block = std::strtoull(argv[3], nullptr, 10);
  try {
    FileReader reader(argv[1], block);
    SimpleFileWriter sink(argv[2]);
    FftSpectrometer<SimpleFileWriter> spec(block, std::strtoull(argv[4], nullptr, 10),
                                           std::strtoull(argv[5], nullptr, 10), std::strtoull(argv[6], nullptr, 10),
                                           1.f, 1.f, sink);
    DadaInputStream<FftSpectrometer<SimpleFileWriter>, FileReader> stream(reader, spec);
    std::printf("blocks %zu\n", stream.start());
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
