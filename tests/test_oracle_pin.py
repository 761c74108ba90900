"""Pins the oracle against the reference's own code and known answers.

* golden fixtures made by the reference's C reference functions compiled from
  its sources (tests/golden/make_golden.py, oracle/build_ref.sh);
* the live reference library when oracle/_ref was built in this checkout;
* the numeric known answers of the reference's gtests.
"""
import ctypes
import os

import numpy as np
import pytest

from oracle import gspec_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
GOLD = os.path.join(HERE, "golden")
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "libref_host.so")


def test_unpack_matches_reference_fixture():
    """Unpacker C references (edd/test/src/UnpackerTester.cu:41-201), bit-exact."""
    g = np.load(os.path.join(GOLD, "ref_unpack.npz"))
    for nbits in (8, 10, 12):
        words = g[f"words{nbits}"]
        ref = g[f"samples{nbits}"]
        got = O.unpack(words.view(np.uint8), nbits).astype(np.float32)
        assert got.shape == ref.shape
        assert np.array_equal(got, ref), nbits


@pytest.mark.skipif(not os.path.exists(REF_LIB), reason="reference library not built (oracle/build_ref.sh)")
def test_unpack_matches_live_reference():
    lib = ctypes.CDLL(REF_LIB)
    lib.ref_unpack.restype = ctypes.c_size_t
    lib.ref_unpack.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int, ctypes.c_void_p]
    rng = np.random.default_rng(99)
    for nbits, mult in ((8, 7), (10, 5), (12, 9)):
        words = rng.integers(0, 2 ** 64, size=mult * 40, dtype=np.uint64)
        words[:8] = [0, 2 ** 64 - 1, 0x8000000000000000, 0x7FFFFFFFFFFFFFFF, 0x0123456789ABCDEF,
                     0xFEDCBA9876543210, 0x8008008008008008, 0x7FF7FF7FF7FF7FF7]
        buf = np.zeros(words.size * 64 // nbits + 64, np.float32)
        n = lib.ref_unpack(words.ctypes.data, words.size, nbits, buf.ctypes.data)
        got = O.unpack(words.view(np.uint8), nbits).astype(np.float32)
        assert np.array_equal(got, buf[:n]), nbits


def test_pack_unpack_roundtrip():
    rng = np.random.default_rng(3)
    for nbits in (8, 10, 12):
        lo, hi = -(1 << (nbits - 1)), (1 << (nbits - 1))
        s = rng.integers(lo, hi, size=4096)
        assert np.array_equal(O.unpack(O.pack(s, nbits), nbits), s)


def test_stokes_known_states():
    """The seven polarisation states of edd/test/src/GatedSpectrometerTest.cu:26-78."""
    g = np.load(os.path.join(GOLD, "ref_stokes.npz"))
    for inp, ref, exp in zip(g["inputs"], g["ref"], g["expected"]):
        p1 = np.complex128(inp[0] + 1j * inp[1])
        p2 = np.complex128(inp[2] + 1j * inp[3])
        got = np.array(O.stokes_iquv(np.array([p1]), np.array([p2]))).ravel()
        np.testing.assert_allclose(got, exp, atol=1e-6)   # EXPECT_FLOAT_EQ values
        np.testing.assert_allclose(got, ref, atol=1e-6)   # reference stokes_IQUV output


def test_detect_matches_reference_fixture():
    """Detector arithmetic: sum over tscrunch of x^2 + y^2 in double
    (edd/test/src/DetectorAccumulatorTester.cu:33-62, the int8 form)."""
    g = np.load(os.path.join(GOLD, "ref_detect.npz"))
    x, nchans, ts, scale = g["x"], int(g["nchans"]), int(g["tscrunch"]), float(g["scale"])
    p = (x[:, 0].astype(np.float64) ** 2 + x[:, 1].astype(np.float64) ** 2)
    # C reference sums float products: x.x * x.x is a float product then promoted
    pf = (x[:, 0] * x[:, 0]).astype(np.float64) + (x[:, 1] * x[:, 1]).astype(np.float64)
    acc = pf.reshape(-1, ts, nchans).sum(axis=1)
    got = ((acc - 0.0) / np.float32(scale)).astype(np.int64).astype(np.int8).ravel()
    assert np.array_equal(got, g["out"])
    assert np.allclose(p.reshape(-1, ts, nchans).sum(axis=1), acc, rtol=1e-6)


def test_gating_known_answers():
    """edd/test/src/GatedSpectrometerTest.cu:142-240: 16 Mi samples of 42 with
    all items 0 (G0 keeps the data, G1 = baseline -4) and all items 1
    (G0 = baseline 5, G1 keeps the data), counts and baseline sums."""
    n = 16 * 1024 * 1024
    v = np.full(n, 42, np.int64)
    items = np.zeros(n, np.uint64)
    g0, g1, m0, m1 = O.gate(v, items, 0, np.float32(-3), np.float32(-4))
    assert np.all(g0 == 42) and np.all(g1 == -4)
    assert m0.sum() == n and m1.sum() == 0
    assert np.sum(v * m0) / m0.sum() == 42.0
    items[:] = 1
    g0, g1, m0, m1 = O.gate(v, items, 0, np.float32(5), np.float32(-2))
    assert np.all(g0 == 5) and np.all(g1 == 42)
    assert m0.sum() == 0 and m1.sum() == n
    assert np.sum(v * m1) / m1.sum() == 42.0
    assert O.baseline(0, 0) == 0.0          # the zero-count guard


def test_gate_float_formula_is_not_identity():
    """(v - b) + b is evaluated in float32 as the reference does; it differs
    from v for some baselines, and the oracle keeps that difference."""
    v = np.arange(-2048, 2048)
    b = np.float32(0.1)
    g0, _, _, _ = O.gate(v, np.zeros(v.size, np.uint64), 0, b, b)
    direct = (v.astype(np.float32) - b) + b
    assert np.array_equal(g0, direct.astype(np.float32))


def test_bit_macros():
    """BitManipulationMacros (edd/test/src/GatedSpectrometerTest.cu:11-23) as
    the gate uses them: bit i of 1<<i is the only set bit."""
    for i in range(63):
        item = np.array([1 << i], np.uint64)
        for j in range(63):
            _, _, m0, m1 = O.gate(np.array([1]), item, j, np.float32(0), np.float32(0))
            assert bool(m1[0]) == (i == j)
    # bit 63 marks a lost heap: neither gate
    _, _, m0, m1 = O.gate(np.array([1]), np.array([1 << 63], np.uint64), 0, np.float32(0), np.float32(0))
    assert not m0[0] and not m1[0]
