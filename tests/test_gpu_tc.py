"""Tensor-core split-precision DFT-1024 (tcgen05, BF16 / FP16 hi+lo halves,
FP32 accumulate) against numpy's FP64 FFT."""
import numpy as np
import pytest

import psrdada_cpp_gb300 as G

pytestmark = pytest.mark.gpu

# BF16 in three parts (bf16x6) and FP16 in two (11-bit mantissas) both leave
# ~2^-22..2^-24 of the spectrum's rms per bin
TOL = {G.FORM_BF16: 1e-5, G.FORM_FP16: 1e-5}


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


# ---------------------------------------------------------------- whole chain
from psrdada_cpp_gb300 import synth  # noqa: E402
from tests.gpu_helpers import run_both  # noqa: E402

S = synth.StreamSpec
# split-precision forms against the FP64 oracle: per-bin relative error (Stokes
# products normalised by I, floor 1 % of the mean) within CHAIN_TOL (max) and
# CHAIN_RMS (root mean square); counters, gate assignment and baselines
# bit-exact as in the FP32 form.  The BF16 form's operands are split in three
# 8-bit parts (bf16x6) and the FP16 form's in two 11-bit parts: both keep
# ~2^-22..2^-24 of each value through the four DFT-32 stages.
CHAIN_TOL = {G.FORM_BF16: 1e-4, G.FORM_FP16: 1e-4}
CHAIN_RMS = {G.FORM_BF16: 1e-5, G.FORM_FP16: 1e-5}
TC_CASES = [
    # dual-pol 12-bit at 2^20 (both passes on the tensor cores), outliers at full scale
    ("d12_n2p20", S("d12_n2p20", 12, True, 6144, 1, 1 << 21, 1 << 20, 2, diode_period_heaps=64), "c3"),
    # single-pol 8-bit at 2^17: N1 = 1024 (pass A on the tensor cores), N2 = 128
    ("s8_n2p17", S("s8_n2p17", 8, False, 4096, 1, 1 << 18, 1 << 17, 2, diode_period_heaps=5), "default"),
    # dual-pol 10-bit at 2^16: N1 = 64, N2 = 1024 (pass B on the tensor cores), 2 blocks per output
    ("d10_n2p16_nb2", S("d10_n2p16", 10, True, 5120, 1, 1 << 16, 1 << 16, 2, diode_period_heaps=3), "default"),
]


@pytest.mark.parametrize("form", [G.FORM_BF16, G.FORM_FP16])
@pytest.mark.parametrize("name,spec,kind", TC_CASES, ids=[c[0] for c in TC_CASES])
def test_tc_chain_matches_oracle(name, spec, kind, form):
    from oracle import gspec_oracle as O
    from tests.gpu_helpers import oracle_config, FLOOR
    prod = {}
    blocks, payloads, worst = run_both(spec, nblocks=6, kind=kind, lost=0.02, form=form, by_product=prod)
    assert payloads, "no output block compared"
    cfg = oracle_config(spec, "intended")
    rms = max(O.rel_err(O.parse_output(bytes(b[:cfg.output_bytes]), cfg)[0], p["spec"], FLOOR, rms=True)
              for b, p in zip(blocks, payloads))
    print(f"{name} form={form} max rel err {worst:.3e} rms {rms:.3e} by product {prod}")
    assert worst <= CHAIN_TOL[form], (worst, prod)
    assert rms <= CHAIN_RMS[form], rms


def test_tc_form_rejected_without_1024_pass():
    lay = G.DadaBufferLayout(4096 * 16 + 16 * 8, 4096, 1)
    with pytest.raises(G.GspecError):
        G.GatedSpectrometer(lay, 0, 0, 4096, 4, 8, 1.0, 1.0, G.NullSink(), form=G.FORM_BF16)
