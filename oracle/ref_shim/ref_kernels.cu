// Device code of the reference's unpack, side-channel merge, gating and Stokes
// kernels, compiled from the reference's own source files where they lie
// (oracle/build_ref.sh) into one sm_103a module, oracle/_ref/ref_kernels.cubin.
// The GPU pin test (tests/test_gpu_ref_kernels.py) loads it through the driver
// API and runs the kernels beside this library's stages.  Test infrastructure
// only: nothing in the library loads it.
#include "psrdada_cpp/effelsberg/edd/src/Unpacker.cu"
#include "psrdada_cpp/effelsberg/edd/src/GatedSpectrometer.cu"
