// Link-time stand-ins for DadaBufferLayout's getters.  The reference defines
// them in edd/src/DadaBufferLayout.cpp, which needs a live psrdada ring
// buffer; they are referenced only by the reference's device-path classes in
// edd/src/GatedSpectrometer.cu, which the pin library never calls.
#include <cstddef>
#include "psrdada_cpp/effelsberg/edd/DadaBufferLayout.hpp"

namespace psrdada_cpp { namespace effelsberg { namespace edd {
size_t DadaBufferLayout::sizeOfData() const { return 0; }
size_t DadaBufferLayout::getHeapSize() const { return 0; }
size_t DadaBufferLayout::getNSideChannels() const { return 0; }
size_t DadaBufferLayout::sizeOfSideChannelData() const { return 0; }
size_t DadaBufferLayout::getNHeaps() const { return 0; }
size_t DadaBufferLayout::sizeOfGap() const { return 0; }
}}}
