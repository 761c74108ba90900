"""Ring-buffer sources and sinks (the steps either side of the path) on the
CPU: the C++ MemoryRing / FileReader / DadaInputStream / DadaOutputStream /
SimpleFileWriter self-test, the psrdada ring clients compiled against
declaration stubs, the Python mirror's reader/writer protocol, and the
gated-file reader against the oracle's output layout."""
import os
import shutil
import subprocess
import threading

import numpy as np
import pytest

from psrdada_cpp_gb300 import ring, gated_file
from psrdada_cpp_gb300.gated_spectrometer import RawBytes, CollectingSink, SimpleFileWriter

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INC = os.path.join(ROOT, "include")
CPP = os.path.join(ROOT, "tests", "cpp")


def _lib_dir():
    from psrdada_cpp_gb300.gated_spectrometer import LIB_PATH
    if not LIB_PATH.exists():
        from psrdada_cpp_gb300.build import build
        build()
    return str(LIB_PATH.parent)


@pytest.mark.skipif(not shutil.which("g++"), reason="no g++")
def test_cpp_ring_selftest(tmp_path):
    exe = str(tmp_path / "selftest")
    lib = _lib_dir()
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", INC,
                        os.path.join(CPP, "ring_selftest.cpp"), "-o", exe, "-L", lib, "-lgspec",
                        "-Wl,-rpath," + lib, "-lpthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, str(tmp_path / "out.dat")], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0 and r.stdout.startswith("ok 37"), r.stdout + r.stderr


@pytest.mark.skipif(not shutil.which("g++"), reason="no g++")
def test_psrdada_clients_compile_against_stubs():
    """The HAVE_PSRDADA clients, compiled against declaration-only stand-ins
    of psrdada's headers (psrdada is not installed)."""
    src = "#include \"psrdada_cpp_gb300/ring.hpp\"\n" \
          "int main() { using namespace psrdada_cpp_gb300;\n" \
          "  PsrdadaReadClient r(0xdada); NullSink s;\n" \
          "  DadaInputStream<NullSink, PsrdadaReadClient> in(r, s); in.start();\n" \
          "  PsrdadaWriteClient w(0xdadb); DadaOutputStream<PsrdadaWriteClient> out(w); (void)out; }\n"
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-DHAVE_PSRDADA", "-I", INC,
                        "-I", os.path.join(CPP, "psrdada_stub"), "-x", "c++", "-"], input=src,
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_memory_ring_protocol():
    rg = ring.MemoryRing(64, 2)
    w, r = rg.writer(), rg.reader()
    got = []

    def produce():
        import ctypes
        h = w.header_stream().next()
        hdr = np.frombuffer(b"HEADER x\n", np.uint8)
        ctypes.memmove(h.ptr(), hdr.ctypes.data, hdr.size)
        h.used_bytes(hdr.size)
        w.header_stream().release()
        for k in range(9):
            b = w.data_stream().next()
            data = np.full(64 - k % 2, k, np.uint8)
            ctypes.memmove(b.ptr(), data.ctypes.data, data.size)
            b.used_bytes(data.size)
            w.data_stream().release()
        w.data_stream().end_of_data()

    class H:
        def init(self, b):
            got.append(bytes(b.numpy()))

        def __call__(self, b):
            got.append(b.numpy().copy())
            return False

    t = threading.Thread(target=produce)
    t.start()
    n = ring.DadaInputStream(r, H()).start()
    t.join()
    assert n == 9 and got[0] == b"HEADER x\n"
    for k in range(9):
        assert got[1 + k].size == 64 - k % 2 and (got[1 + k] == k).all()
    with pytest.raises(RuntimeError):
        r.data_stream().release()          # nothing acquired
    with pytest.raises(RuntimeError):
        r.data_stream().next()             # end of data, no block


def test_output_stream_and_file_reader(tmp_path):
    """DadaOutputStream copies into a ring; SimpleFileWriter + FileReader
    round-trip whole blocks."""
    rg = ring.MemoryRing(32, 4)
    out = ring.DadaOutputStream(rg.writer())
    hdr = np.zeros(4096, np.uint8)
    hdr[:7] = np.frombuffer(b"HEADER\n", np.uint8)
    out.init(RawBytes(hdr))
    blocks = [np.arange(32, dtype=np.uint8) + k for k in range(3)]
    for b in blocks:
        out(RawBytes(b))
    rg.writer().data_stream().end_of_data()
    path = str(tmp_path / "f.dada")
    sink = SimpleFileWriter(path)
    assert ring.DadaInputStream(rg.reader(), sink).start() == 3
    sink.close()
    assert os.path.getsize(path) == 4096 + 3 * 32
    col = CollectingSink()
    fr = ring.FileReader(path, 32)
    assert ring.DadaInputStream(fr, col).start() == 3
    fr.close()
    assert col.header[:7] == b"HEADER\n"
    for a, b in zip(col.blocks, blocks):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("dual", [False, True])
def test_gated_file_reader_layout(tmp_path, dual):
    """The reader parses a file in the reference output layout (made by the
    oracle's layout writer): spectra, both counters per row, header keys."""
    from oracle import gspec_oracle as O
    rng = np.random.default_rng(3)
    C, n_out = 33, 5
    spec = rng.random((n_out, 4, 2, C) if dual else (n_out, 2, C)) * 1e6
    n0 = rng.integers(0, 1 << 40, n_out, dtype=np.uint64)
    n1 = rng.integers(0, 1 << 40, n_out, dtype=np.uint64)
    body = O.output_bytes(spec, n0, n1, dual)
    hdr = bytearray(b"HEADER DADA\n")
    cfg_text = O.HEADER_PARAM_FMT.format(fft=64, nchans=C, nacc=8, sel=0, bit=0, stokes="yes" if dual else "no")
    hdr += cfg_text.encode()
    hdr = bytes(hdr).ljust(4096, b"\0")
    path = tmp_path / "g.dat"
    path.write_bytes(hdr + body + body)
    g = gated_file.read_gated_file(str(path))
    assert g.fft_length == 64 and g.nchans == C and g.naccumulate == 8 and g.stokes == dual
    assert g.rows == 2 * n_out and g.trailing_bytes == 0
    assert np.array_equal(g.n0, np.tile(n0, 2)) and np.array_equal(g.n1, np.tile(n1, 2))
    assert np.array_equal(g.spectra[:n_out], spec.astype(np.float32).astype(np.float64))
    if dual:
        assert np.array_equal(g.stokes_product("U", 1), g.spectra[:, 2, 1])
