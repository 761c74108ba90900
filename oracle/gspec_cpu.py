"""ctypes wrapper of oracle/libgspec_cpu.so, the C/OpenMP restatement of the
chain (TEST AND CPU-BASELINE INFRASTRUCTURE ONLY: imported by tests/ and by
bench.py's CPU legs)."""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libgspec_cpu.so")


class CpuCfg(ctypes.Structure):
    _fields_ = [(n, ctypes.c_uint64) for n in (
        "buffer_size", "heap_size", "nsc", "sel", "bitpos", "fft_length", "naccumulate")] + \
        [(n, ctypes.c_uint32) for n in ("nbits", "dual", "convention")] + \
        [(n, ctypes.c_uint64) for n in (
            "n_heaps", "gap", "data_bytes", "sc_off", "nsamps", "items_per_pol", "n_blocks", "batch", "nacc",
            "n_out", "C", "rec")]


_lib = None


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            subprocess.run(["bash", os.path.join(HERE, "build_cpu.sh")], check=True)
        lib = ctypes.CDLL(LIB)
        lib.cpu_configure.argtypes = [ctypes.POINTER(CpuCfg)]
        lib.cpu_run_block.argtypes = [ctypes.POINTER(CpuCfg), ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_void_p, ctypes.c_int]
        lib.cpu_max_threads.restype = ctypes.c_int
        _lib = lib
    return _lib


def max_threads() -> int:
    return load().cpu_max_threads()


class CpuChain:
    """One stream of the chain on the host: ``run_block`` accumulates one
    block into ``out`` (reference output layout) and updates the baselines."""

    def __init__(self, spec, convention: str = "intended", nthreads: int = 0):
        lib = load()
        c = CpuCfg(buffer_size=spec.buffer_size, heap_size=spec.heap_size, nsc=spec.n_side_channels,
                   sel=spec.selected_side_channel, bitpos=spec.selected_bit, fft_length=spec.fft_length,
                   naccumulate=spec.naccumulate, nbits=spec.nbits, dual=int(spec.dual_pol),
                   convention=1 if convention == "reference" else 0)
        rc = lib.cpu_configure(ctypes.byref(c))
        if rc != 0:
            raise ValueError(f"cpu_configure failed ({rc})")
        self.cfg = c
        self.nthreads = nthreads
        self.baselines = np.zeros(4, np.float32)
        self.out = np.zeros(c.rec * c.n_out, np.uint8)
        self.sat = np.zeros(2 * c.n_out, np.uint64)

    def zero(self):
        self.out[:] = 0
        self.sat[:] = 0

    def run_block(self, block: np.ndarray):
        block = np.ascontiguousarray(block, dtype=np.uint8)
        rc = load().cpu_run_block(ctypes.byref(self.cfg), block.ctypes.data, self.out.ctypes.data,
                                  self.sat.ctypes.data, self.baselines.ctypes.data, self.nthreads)
        if rc != 0:
            raise RuntimeError(f"cpu_run_block failed ({rc})")
