"""Tensor-core split-precision DFT-1024 (tcgen05, BF16 / FP16 hi+lo halves,
FP32 accumulate) against numpy's FP64 FFT."""
import numpy as np
import pytest

import psrdada_cpp_gb300 as G

pytestmark = pytest.mark.gpu

# BF16 hi+lo: the dropped lo*lo term and the FP32 accumulation leave ~1e-5 of
# the spectrum's rms per bin; FP16 halves (11-bit mantissas) ~1e-7
TOL = {G.FORM_BF16: 1e-4, G.FORM_FP16: 1e-5}


def run_tc(x: np.ndarray, form: int) -> np.ndarray:
    import torch
    dev = torch.device("cuda", 0)
    d_in = torch.from_numpy(x.astype(np.complex64).view(np.float32)).to(dev)
    d_out = torch.zeros_like(d_in)
    G.tc_dft1024_device(d_in.data_ptr(), d_out.data_ptr(), x.shape[0], form)
    torch.cuda.synchronize(dev)
    return d_out.cpu().numpy().view(np.complex64).reshape(x.shape)


@pytest.mark.parametrize("form", [G.FORM_BF16, G.FORM_FP16])
def test_tc_dft1024_matches_fp64(form):
    rng = np.random.default_rng(5)
    x = (rng.normal(0, 300, (16, 1024)) + 1j * rng.normal(0, 300, (16, 1024)))
    if form == G.FORM_FP16:
        x = x / 64.0                                      # FP16 range: |X| <= 1024 max|x|
    x = x.astype(np.complex64)
    got = run_tc(x, form).astype(np.complex128)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    err = np.abs(got - ref) / np.sqrt(np.mean(np.abs(ref) ** 2, axis=1, keepdims=True))
    assert err.max() < TOL[form], err.max()


def test_tc_dft1024_tones_and_impulse():
    n = np.arange(1024)
    x = np.zeros((4, 1024), np.complex64)
    x[0, 0] = 1000.0                                      # impulse -> flat spectrum
    x[1] = 100.0 * np.exp(2j * np.pi * 5 * n / 1024)       # tone at bin 5
    x[2] = 100.0 * np.exp(-2j * np.pi * 1000 * n / 1024)   # tone at bin 24
    x[3] = 50.0                                           # DC
    got = run_tc(x, G.FORM_BF16)
    ref = np.fft.fft(x.astype(np.complex128), axis=1)
    scale = np.abs(ref).max(axis=1, keepdims=True)
    assert (np.abs(got - ref) / scale).max() < 1e-4
    assert np.argmax(np.abs(got[1])) == 5 and np.argmax(np.abs(got[2])) == 24
