"""VLBI on the GPU (gspec_vlbi_*, the VLBI<Handler> drop-in) against the
oracle: every handed-out buffer of VDIF frames byte-equal to OracleVLBI's,
for 8- and 12-bit samples, frames that straddle blocks (spill-over), a first
second that starts inside the first block and one that skips whole blocks;
the C++ drop-in in the reference's CLI wiring gives the same bytes."""
import os
import subprocess

import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth
from psrdada_cpp_gb300.vlbi import VLBI, VDIFHeader
import psrdada_cpp_gb300 as G

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header(sync_time, clock_start):
    h = np.zeros(4096, np.uint8)
    t = (f"HEADER       DADA\nHDR_VERSION  1.0\nSYNC_TIME    {sync_time}\n"
         f"SAMPLE_CLOCK_START {clock_start}\n").encode()
    h[:len(t)] = np.frombuffer(t, np.uint8)
    return h


def _blocks(nbits, nsamp, n, seed):
    out = []
    for b in range(n):
        rng = np.random.default_rng([seed, b])
        x = np.clip(np.rint(rng.normal(3.0, 0.3 * (1 << (nbits - 1)) / 3, nsamp)),
                    -(1 << (nbits - 1)), (1 << (nbits - 1)) - 1).astype(np.int64)
        out.append(synth.pack_samples(x, nbits))
    return out


# (nbits, samples per block, frame length in 8-byte units, sample rate, SAMPLE_CLOCK_START)
CASES = [(8, 1 << 16, 129, 4096.0 * 64, 5000),          # 1000-byte payload: frames straddle blocks
         (12, 1 << 16, 253, 2016.0 * 4 * 9, 70000),     # the first second starts inside block 1
         (8, 1 << 14, 36, 1.0e6, 3)]                    # ~1 s to skip: whole blocks dropped


@pytest.mark.parametrize("nbits,nsamp,flen,rate,clock", CASES, ids=["b8_spill", "b12_skip", "b8_drop"])
def test_vlbi_matches_oracle(nbits, nsamp, flen, rate, clock):
    blocks = _blocks(nbits, nsamp, 12 if clock > 100 else 80, seed=flen)
    nbytes = blocks[0].size
    hdr = VDIFHeader()
    hdr.setDataFrameLength(flen)
    hdr.setStationId(0x4566)
    sink = G.CollectingSink()
    orc = O.OracleVLBI(nbytes, nbits, rate, 0.981599, hdr.getData())
    orc.init(1700000000, clock)
    refs = [x for x in (orc(b)[1] for b in blocks) if x is not None]
    with VLBI(nbytes, nbits, 4096, rate, 0.981599, hdr, sink) as v:
        h = _header(1700000000, clock)
        v.init(G.RawBytes(h))
        assert b"# VLBI parameters:" in bytes(sink.header)
        for b in blocks:
            assert v(G.RawBytes(b)) is False
        info = v.info()
    assert refs and len(sink.blocks) == len(refs)
    for i, (got, ref) in enumerate(zip(sink.blocks, refs)):
        assert got.size == info.output_bytes
        assert bytes(got) == ref, f"output {i} differs"
    # the frames are 2-bit, valid, and carry the station id
    w = np.frombuffer(refs[0][:32], "<u4")
    assert (w[3] >> 26) & 0x1F == 1 and w[3] & 0xFFFF == 0x4566 and not (w[0] >> 31)


def test_vlbi_cpp_drop_in(tmp_path):
    G.load_library()
    pkg = os.path.join(ROOT, "psrdada_cpp_gb300")
    exe = str(tmp_path / "vlbi_pipeline")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "vlbi_pipeline.cpp"), "-o", exe, "-L", pkg, "-lgspec",
                        "-Wl,-rpath," + pkg, "-lpthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nbits, nsamp, flen, rate, clock = 8, 1 << 16, 129, 4096.0 * 64, 5000
    blocks = _blocks(nbits, nsamp, 9, seed=3)
    path = tmp_path / "in.dada"
    path.write_bytes(_header(1700000000, clock).tobytes() + b"".join(b.tobytes() for b in blocks))
    outp = tmp_path / "out.vdif"
    r = subprocess.run([exe, str(path), str(outp), str(blocks[0].size), str(nbits), str(rate), "0.981599",
                        str(flen), str(0x4566)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0 and "blocks 9" in r.stdout, r.stdout + r.stderr
    hdr = VDIFHeader()
    hdr.setDataFrameLength(flen)
    hdr.setStationId(0x4566)
    hdr.setNumberOfChannels(0)
    orc = O.OracleVLBI(blocks[0].size, nbits, rate, 0.981599, hdr.getData())
    orc.init(1700000000, clock)
    refs = [x for x in (orc(b)[1] for b in blocks) if x is not None]
    data = outp.read_bytes()
    assert data[4096:] == b"".join(refs)
