"""VLBI on the CPU: VDIF time fields from the C ABI against the calendar,
header accessors, the oracle's frame stream, configuration errors before any
CUDA call, and the C++ drop-in compiling."""
import ctypes
import datetime
import os
import shutil
import subprocess

import numpy as np
import pytest

from oracle import gspec_oracle as O

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("when", ["2000-01-01T00:00:00", "2019-06-30T23:59:59", "2019-07-01T00:00:00",
                                  "2024-02-29T12:34:56", "2026-12-04T13:46:32"])
def test_vdif_time_fields(when):
    from psrdada_cpp_gb300.vlbi import VDIFHeader
    t = int(datetime.datetime.fromisoformat(when).replace(tzinfo=datetime.timezone.utc).timestamp())
    h = VDIFHeader()
    h.setTimeReferencesFromTimestamp(t)
    ep, sec = O.vdif_time_fields(t)
    assert (h.getReferenceEpoch(), h.getSecondsFromReferenceEpoch()) == (ep, sec)
    assert h.getTimestamp() == t


def test_vdif_header_fields():
    from psrdada_cpp_gb300.vlbi import VDIFHeader
    h = VDIFHeader()
    assert h.getVersionNumber() == 1 and h.isValid() and h.isRealDataType()
    h.setDataFrameLength(1004)
    h.setStationId(0x4566)
    h.setThreadId(3)
    h.setBitsPerSample(1)
    h.setDataFrameNumber(12345)
    h.setInvalid()
    assert (h.getDataFrameLength(), h.getStationId(), h.getThreadId(), h.getBitsPerSample(),
            h.getDataFrameNumber()) == (1004, 0x4566, 3, 1, 12345)
    assert not h.isValid()
    with pytest.raises(ValueError):
        h.setThreadId(1 << 10)
    with pytest.raises(ValueError):
        VDIFHeader().setTimeReferencesFromTimestamp(946684799)   # before 2000


def test_oracle_frames_carry_the_stream():
    """Valid payloads of consecutive outputs concatenate to the 2-bit stream
    after the skip; frame numbers advance and wrap at frames per second."""
    rng = np.random.default_rng(1)
    nbits, nbytes = 8, 16000                        # 4000 2-bit bytes per block: more than the skip
    blocks = [rng.integers(-100, 100, nbytes).astype(np.int8).view(np.uint8) for _ in range(8)]
    hdr = [0] * 8
    hdr[2] = 124 | (1 << 29)                       # 992-byte frames: 960 payload bytes
    o = O.OracleVLBI(nbytes, nbits, 960 * 4 * 3.0, 0.98, hdr)   # 3 frames per second
    o.init(1500000000, 7)                          # a fraction of a second to skip
    skip = o.skip
    outs = [x for x in (o(b)[1] for b in blocks) if x is not None]
    assert len(outs) == 5
    payload = b""
    nums = []
    for out in outs:
        for f in range(o.nframes):
            w = np.frombuffer(out[f * 992:f * 992 + 32], "<u4")
            if not (w[0] >> 31):
                payload += out[f * 992 + 32:(f + 1) * 992]
                nums.append(int(w[1]) & 0xFFFFFF)
    stream = b"".join(O.vlbi_pack2bit(O.unpack(b, nbits), 0.98).tobytes() for b in blocks[:5])[skip:]
    assert payload == stream[:len(payload)] and len(payload) > 0
    assert nums == [i % 3 for i in range(len(nums))]


def test_vlbi_configuration_errors_without_gpu():
    from psrdada_cpp_gb300.vlbi import GspecVlbiConfig, _lib
    lib = _lib()
    err = ctypes.create_string_buffer(256)

    def create(**kw):
        c = GspecVlbiConfig(buffer_size=4096, nbits=8, sample_rate=1e6, digitizer_threshold=0.98)
        c.vdif_header[2] = 100
        for k, v in kw.items():
            if k == "frame_len":
                c.vdif_header[2] = v
            else:
                setattr(c, k, v)
        h = lib.gspec_vlbi_create(ctypes.byref(c), err, 256)
        if h:
            lib.gspec_vlbi_destroy(h)
            return None
        return err.value.decode()

    assert "nbits" in create(nbits=10)
    assert "frame length" in create(frame_len=4)
    assert "threshold" in create(digitizer_threshold=0.0)
    assert "one VDIF frame per second" in create(sample_rate=10.0)


@pytest.mark.skipif(not shutil.which("g++"), reason="no g++")
def test_cpp_vlbi_compiles():
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "vlbi_pipeline.cpp")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
