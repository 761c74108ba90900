"""The reference's own GPU kernels - Unpacker's unpack_edd_{8,12}bit_to_float32
(psrdada_cpp/effelsberg/edd/src/Unpacker.cu:24-108), mergeSideChannels, gating
and stokes_accumulate (psrdada_cpp/effelsberg/edd/src/GatedSpectrometer.cu:9-90,
140-169) - loaded from oracle/_ref/ref_kernels.cubin (compiled from the
reference's source files by oracle/build_ref.sh) and launched through the CUDA
driver API with ctypes, with the launch shapes of the reference's own call
sites (edd/src/Unpacker.cu:124-140, edd/detail/GatedSpectrometer.cu:243-251,
398-425).  Test infrastructure: a second pin of this library's stages."""
from __future__ import annotations

import ctypes
import os

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUBIN = os.path.join(ROOT, "oracle", "_ref", "ref_kernels.cubin")
NAMES = os.path.join(ROOT, "oracle", "_ref", "ref_kernels.names")

# kernel -> a token of its symbol name (Itanium mangling of the reference's declarations)
TOKENS = {
    "unpack8": "26unpack_edd_8bit_to_float32",
    "unpack12": "27unpack_edd_12bit_to_float32",
    "merge": "17mergeSideChannels",
    "gating": "6gatingE",
    "stokes": "17stokes_accumulate",
}


def available() -> bool:
    return os.path.exists(CUBIN) and os.path.exists(NAMES)


class RefKernels:
    """Loads the module into the current context (the caller has initialised
    CUDA on the device, e.g. through torch)."""

    def __init__(self):
        cu = ctypes.CDLL("libcuda.so.1")
        vp = ctypes.c_void_p
        cu.cuCtxGetCurrent.argtypes = [ctypes.POINTER(vp)]
        cu.cuModuleLoad.argtypes = [ctypes.POINTER(vp), ctypes.c_char_p]
        cu.cuModuleGetFunction.argtypes = [ctypes.POINTER(vp), vp, ctypes.c_char_p]
        cu.cuModuleUnload.argtypes = [vp]
        cu.cuLaunchKernel.argtypes = [vp] + [ctypes.c_uint] * 7 + [vp, ctypes.POINTER(vp), ctypes.POINTER(vp)]
        self.cu = cu
        ctx = vp()
        self._check(cu.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context (initialise the device first)")
        self.mod = vp()
        self._check(cu.cuModuleLoad(ctypes.byref(self.mod), CUBIN.encode()), "cuModuleLoad")
        names = open(NAMES).read().split()
        self.fn = {}
        for key, token in TOKENS.items():
            matches = [n for n in names if token in n]
            if len(matches) != 1:
                raise RuntimeError(f"kernel {key}: {len(matches)} symbols match {token}")
            f = vp()
            self._check(cu.cuModuleGetFunction(ctypes.byref(f), self.mod, matches[0].encode()), key)
            self.fn[key] = f

    @staticmethod
    def _check(rc, what):
        if rc != 0:
            raise RuntimeError(f"{what} failed with CUresult {rc}")

    def launch(self, key: str, grid: int, block: int, args, stream: int = 0):
        """args: ctypes values in the kernel's parameter order."""
        arr = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in args])
        self._check(self.cu.cuLaunchKernel(self.fn[key], grid, 1, 1, block, 1, 1, 0, ctypes.c_void_p(stream),
                                           arr, None), key)

    def close(self):
        if self.mod:
            self.cu.cuModuleUnload(self.mod)
            self.mod = None


def ptr(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


def size(n: int) -> ctypes.c_uint64:
    return ctypes.c_uint64(n)
