"""The ungated FftSpectrometer on the CPU: the oracle's restatement against a
direct DFT on a tone, configuration errors before any CUDA call, and the C++
drop-in header compiling with the reference's type names."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("nbits", [8, 10, 12])
def test_oracle_fft_spectrometer_tone(nbits):
    N, nacc, nf = 64, 4, 8
    n = np.arange(N * nf)
    x = np.rint(20 * np.cos(2 * np.pi * 5 * n / N)).astype(np.int64)
    raw = synth.pack_samples(x, nbits)
    p = O.fft_spectrometer_block(raw, nbits, N, nacc)
    assert p.shape == (nf // nacc, N // 2 + 1)
    ref = (np.abs(np.fft.rfft(x.reshape(nf, N).astype(np.float64), axis=1)) ** 2).reshape(2, nacc, -1).sum(1)
    assert np.allclose(p, ref, rtol=1e-12)
    assert np.argmax(p[0]) == 5


def test_ungated_configuration_errors_without_gpu():
    import ctypes
    from psrdada_cpp_gb300.gated_spectrometer import GspecConfig, load_library, FLAG_UNGATED
    lib = load_library()
    err = ctypes.create_string_buffer(256)

    def create(**kw):
        base = dict(buffer_size=1 << 16, heap_size=0, n_side_channels=0, fft_length=1024, naccumulate=4, nbits=8,
                    flags=FLAG_UNGATED)
        base.update(kw)
        h = lib.gspec_create(ctypes.byref(GspecConfig(**base)), err, 256)
        if h:
            lib.gspec_destroy(h)
            return None
        return err.value.decode()

    assert "n_side_channels" in create(n_side_channels=1)
    assert "single-pol" in create(input_type=1, output_type=1)
    assert "convention" in create(convention=1)
    assert "multiple" in create(naccumulate=3)


@pytest.mark.skipif(not shutil.which("g++"), reason="no g++")
def test_cpp_fft_spectrometer_compiles():
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "fft_pipeline.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
