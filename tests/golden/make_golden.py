"""Generates the golden fixtures in tests/golden/.

  * ref_unpack.npz  - random big-endian words and the samples the
    reference's own C unpackers produce for them
    (edd/test/src/UnpackerTester.cu:41-201, built by oracle/build_ref.sh);
  * ref_stokes.npz  - the seven polarisation states of
    edd/test/src/GatedSpectrometerTest.cu:26-78 evaluated by the reference's
    stokes_IQUV (edd/src/GatedSpectrometer.cu:125-131);
  * ref_detect.npz  - detect_c_reference (edd/test/src/DetectorAccumulatorTester.cu:33-62)
    on seeded input;
  * chain_*.npz     - small end-to-end cases: input blocks and the oracle's
    handler outputs (regression fixtures for the oracle itself).

Run from the repository root after ``bash oracle/build_ref.sh``:
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import gspec_oracle as O  # noqa: E402
from psrdada_cpp_gb300 import synth  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))


def ref_lib():
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libref_host.so"))
    lib.ref_unpack.restype = ctypes.c_size_t
    lib.ref_unpack.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    lib.ref_stokes_iquv.argtypes = [ctypes.c_float] * 4 + [ctypes.c_void_p]
    lib.ref_detect_int8.restype = ctypes.c_size_t
    lib.ref_detect_int8.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_int, ctypes.c_float,
                                    ctypes.c_float, ctypes.c_void_p]
    return lib


STOKES_STATES = {
    # name: (p1, p2) exactly as the reference test writes them
    "no_field": ((0.0, 0.0), (0.0, 0.0)),
    "horizontal": ((1.0, 0.0), (0.0, 0.0)),
    "vertical": ((0.0, 0.0), (1.0, 0.0)),
    "linear_p45": ((float(np.float32(1 / np.sqrt(2))), 0.0), (float(np.float32(1 / np.sqrt(2))), 0.0)),
    "linear_m45": ((float(np.float32(-1 / np.sqrt(2))), 0.0), (float(np.float32(1 / np.sqrt(2))), 0.0)),
    "left_circular": ((0.0, float(np.float32(1 / np.sqrt(2)))), (float(np.float32(1 / np.sqrt(2))), 0.0)),
    "right_circular": ((0.0, float(np.float32(-1 / np.sqrt(2)))), (float(np.float32(1 / np.sqrt(2))), 0.0)),
}
# expected (I, Q, U, V) from the reference test's EXPECT_FLOAT_EQ lines
STOKES_EXPECTED = {
    "no_field": (0, 0, 0, 0), "horizontal": (1, 1, 0, 0), "vertical": (1, -1, 0, 0),
    "linear_p45": (1, 0, 1, 0), "linear_m45": (1, 0, -1, 0), "left_circular": (1, 0, 0, -1),
    "right_circular": (1, 0, 0, 1),
}


def make_ref_fixtures(lib):
    rng = np.random.default_rng(20240601)
    out = {}
    for nbits, mult in ((8, 1), (10, 5), (12, 3)):
        words = rng.integers(0, 2 ** 64, size=mult * 256, dtype=np.uint64)
        buf = np.zeros(words.size * 64 // nbits + 64, np.float32)
        n = lib.ref_unpack(words.ctypes.data, words.size, nbits, buf.ctypes.data)
        out[f"words{nbits}"] = words
        out[f"samples{nbits}"] = buf[:n].copy()
    np.savez_compressed(os.path.join(HERE, "ref_unpack.npz"), **out)

    names = list(STOKES_STATES)
    vals = np.zeros((len(names), 4), np.float32)
    o = np.zeros(4, np.float32)
    for i, nm in enumerate(names):
        (a, b), (c, d) = STOKES_STATES[nm]
        lib.ref_stokes_iquv(a, b, c, d, o.ctypes.data)
        vals[i] = o
    inputs = np.array([[*STOKES_STATES[n][0], *STOKES_STATES[n][1]] for n in names], np.float32)
    expected = np.array([STOKES_EXPECTED[n] for n in names], np.float32)
    np.savez_compressed(os.path.join(HERE, "ref_stokes.npz"), names=np.array(names), inputs=inputs,
                        ref=vals, expected=expected)

    nchans, tscrunch = 64, 16
    x = rng.normal(0, 15.0, size=(nchans * tscrunch * 8, 2)).astype(np.float32)
    det = np.zeros(x.shape[0] // tscrunch, np.int8)
    scale = float(np.sqrt(15.0 * tscrunch))
    n = lib.ref_detect_int8(x.ctypes.data, x.shape[0], nchans, tscrunch, scale, 0.0, det.ctypes.data)
    np.savez_compressed(os.path.join(HERE, "ref_detect.npz"), x=x, out=det[:n], nchans=nchans, tscrunch=tscrunch,
                        scale=scale)


CHAIN_CASES = {
    "chain_single8": dict(spec=synth.StreamSpec("s8", 8, False, 4096, 1, 1 << 15, 256, 16, diode_period_heaps=3),
                          kind="default", convention="intended", nblocks=6, lost=0.1),
    "chain_dual12": dict(spec=synth.StreamSpec("d12", 12, True, 6144, 1, 1 << 14, 512, 8, diode_period_heaps=1),
                         kind="default", convention="intended", nblocks=6, lost=0.1),
    "chain_single8_reference": dict(
        spec=synth.StreamSpec("s8r", 8, False, 4096, 1, 1 << 15, 512, 16, diode_period_heaps=3),
        kind="default", convention="reference", nblocks=5, lost=0.0),
}


def chain_config(spec, convention):
    lay = O.BufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    return O.Config(lay, spec.selected_side_channel, spec.selected_bit, spec.fft_length, spec.naccumulate,
                    spec.nbits, spec.dual_pol, convention)


def make_chain_fixture(name, case):
    spec = case["spec"]
    cfg = chain_config(spec, case["convention"])
    blocks = [synth.make_block(spec, seed=7, block_index=b, kind=case["kind"], lost_frac=case["lost"])
              for b in range(case["nblocks"])]
    orc = O.OracleSpectrometer(cfg)
    outs = []
    for blk in blocks:
        stop, payload = orc(blk)
        if payload is not None:
            outs.append(np.frombuffer(payload["bytes"], np.uint8))
    np.savez_compressed(os.path.join(HERE, name + ".npz"), blocks=np.stack(blocks), outputs=np.stack(outs))


if __name__ == "__main__":
    lib = ref_lib()
    make_ref_fixtures(lib)
    for name, case in CHAIN_CASES.items():
        make_chain_fixture(name, case)
    print("golden fixtures written to", HERE)
