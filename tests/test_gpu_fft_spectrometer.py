"""The ungated FftSpectrometer (edd/detail/FftSpectrometer.cu:13-179) on the
GPU through the C ABI against the oracle: each handed-out block is the
previous-but-two input block's power spectra (the reference's pipeline
delay), n_out x (fft/2 + 1) float32 within the FP32 tolerance; the C++
drop-in in the reference's CLI wiring gives the same bytes."""
import os
import subprocess

import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth
import psrdada_cpp_gb300 as G
from tests.gpu_helpers import SPEC_TOL

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

# (nbits, samples per block, fft_length, naccumulate, kind): the shared-memory
# FFT path and the four-step path, 8/10/12-bit
CASES = [(8, 1 << 18, 1024, 16, "c1"), (12, 1 << 18, 4096, 4, "default"), (10, 1 << 18, 512, 32, "default"),
         (12, 1 << 19, 1 << 16, 2, "c3"), (8, 1 << 20, 1 << 20, 1, "default")]


def _blocks(nbits, nsamp, fft, kind, n=6, seed=31):
    spec = synth.StreamSpec("fftspec", nbits, False, 4096 * nbits // 8, 1, nsamp, fft, 1)
    out = []
    for b in range(n):
        rng = np.random.default_rng([seed, b])
        s = synth.config_samples(spec, rng, kind)[0]
        out.append(synth.pack_samples(s, nbits))
    return out


@pytest.mark.parametrize("nbits,nsamp,fft,nacc,kind", CASES, ids=[f"b{c[0]}_n{c[2]}" for c in CASES])
def test_fft_spectrometer_matches_oracle(nbits, nsamp, fft, nacc, kind):
    blocks = _blocks(nbits, nsamp, fft, kind)
    sink = G.CollectingSink()
    nbytes = blocks[0].size
    with G.FftSpectrometer(nbytes, fft, nacc, nbits, 1.0, 1.0, sink) as fs:
        hdr = np.zeros(4096, np.uint8)
        hdr[:6] = np.frombuffer(b"HEADER", np.uint8)
        fs.init(G.RawBytes(hdr))
        assert bytes(sink.header[:6]) == b"HEADER" and not bytes(sink.header[6:]).strip(b"\0")
        for b in blocks:
            assert fs(G.RawBytes(b)) is False
        n_out = int(fs.info().n_out)
    C = fft // 2 + 1
    # blocks 0..n-4 handed out at calls 4..n, as the reference's pipeline
    assert len(sink.blocks) == len(blocks) - 3
    worst = 0.0
    for i, got in enumerate(sink.blocks):
        assert got.size == n_out * C * 4
        ref = O.fft_spectrometer_block(blocks[i], nbits, fft, nacc)
        worst = max(worst, O.rel_err(got.view("<f4").reshape(n_out, 1, C), ref[:, None, :]))
    print(f"b{nbits} n{fft}: max rel err {worst:.3e}")
    assert worst <= SPEC_TOL


def test_fft_spectrometer_cpp_drop_in(tmp_path):
    G.load_library()
    pkg = os.path.join(ROOT, "psrdada_cpp_gb300")
    exe = str(tmp_path / "fft_pipeline")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "fft_pipeline.cpp"), "-o", exe, "-L", pkg, "-lgspec",
                        "-Wl,-rpath," + pkg, "-lpthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nbits, nsamp, fft, nacc = 8, 1 << 18, 1024, 16
    blocks = _blocks(nbits, nsamp, fft, "c1", n=7, seed=32)
    hdr = np.zeros(4096, np.uint8)
    hdr[:12] = np.frombuffer(b"HEADER DADA\n", np.uint8)
    path = tmp_path / "in.dada"
    path.write_bytes(hdr.tobytes() + b"".join(b.tobytes() for b in blocks))
    outp = tmp_path / "out.dat"
    r = subprocess.run([exe, str(path), str(outp), str(blocks[0].size), str(fft), str(nacc), str(nbits)],
                       capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "blocks 7" in r.stdout, r.stdout + r.stderr
    sink = G.CollectingSink()
    with G.FftSpectrometer(blocks[0].size, fft, nacc, nbits, 1.0, 1.0, sink) as fs:
        for b in blocks:
            fs(G.RawBytes(b))
    data = outp.read_bytes()
    assert data[:4096] == hdr.tobytes()
    assert data[4096:] == b"".join(x.tobytes() for x in sink.blocks)


def test_fft_spectrometer_rejects_gated_settings():
    with pytest.raises(G.GspecError, match="n_side_channels"):
        lay = G.DadaBufferLayout(1 << 16, 4096, 1)
        G.GatedSpectrometer(lay, 0, 0, 1024, 4, 8, 1.0, 1.0, G.NullSink(), flags=G.FLAG_UNGATED)
    with pytest.raises(G.GspecError, match="single-pol"):
        lay = G.DadaBufferLayout(1 << 16, 1 << 16, 0)
        G.GatedSpectrometer(lay, 0, 0, 1024, 4, 8, 1.0, 1.0, G.NullSink(), input_type=G.DUAL_POL,
                            flags=G.FLAG_UNGATED)
