// VLBI in the reference's CLI wiring (edd/src/VLBI_cli.cu: DadaInputStream ->
// VLBI -> sink), reading a DADA file through FileReader and writing the
// VDIF frames with SimpleFileWriter.
//
//   vlbi_pipeline <in.dada> <out.vdif> <block_bytes> <nbits> <sample_rate> <threshold> <frame_len_8B> <station>
#include <cstdio>
#include <cstdlib>
#include <iostream>

#include "psrdada_cpp_gb300/VLBI.hpp"
#include "psrdada_cpp_gb300/ring.hpp"

using namespace psrdada_cpp_gb300;

int main(int argc, char** argv) {
  if (argc < 9) {
    std::cerr << "usage: " << argv[0] << " in out block_bytes nbits rate threshold frame_len station\n";
    return 2;
  }
  const std::size_t block = std::strtoull(argv[3], nullptr, 10);
  try {
    VDIFHeader header;
    header.setDataFrameLength(static_cast<uint32_t>(std::strtoul(argv[7], nullptr, 10)));
    header.setStationId(static_cast<uint32_t>(std::strtoul(argv[8], nullptr, 10)));
    header.setNumberOfChannels(0);
    FileReader reader(argv[1], block);
    SimpleFileWriter sink(argv[2]);
    VLBI<SimpleFileWriter> vlbi(block, std::strtoull(argv[4], nullptr, 10), 4096, std::strtod(argv[5], nullptr),
                                std::strtod(argv[6], nullptr), header, sink);
    DadaInputStream<VLBI<SimpleFileWriter>, FileReader> stream(reader, vlbi);
    std::printf("blocks %zu output_bytes %llu\n", stream.start(),
                static_cast<unsigned long long>(vlbi.info().output_bytes));
  } catch (const std::exception& e) {
    std::cerr << "error: " << e.what() << "\n";
    return 1;
  }
  return 0;
}
