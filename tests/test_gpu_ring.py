"""The spectrometer between rings on the GPU: DADA blocks from a page-locked
input ring through DadaInputStream -> GatedSpectrometer -> DadaOutputStream
into an output ring and a file, in C++ (tests/cpp/ring_pipeline.cpp) and in
the Python mirror; every output byte equals the direct handler calls, and the
file read back with the gated-file reader matches the oracle."""
import os
import subprocess
import threading

import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth, ring, gated_file
import psrdada_cpp_gb300 as G
from tests.gpu_helpers import oracle_config, SPEC_TOL

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
S = synth.StreamSpec
CASES = [S("ring_s8", 8, False, 4096, 1, 1 << 15, 512, 8, diode_period_heaps=2),
         S("ring_d12", 12, True, 6144, 1, 1 << 16, 16384, 2, diode_period_heaps=3)]


def _header():
    h = np.zeros(4096, np.uint8)
    t = b"HEADER       DADA\nHDR_VERSION  1.0\nHDR_SIZE     4096\n"
    h[:len(t)] = np.frombuffer(t, np.uint8)
    return h


def _direct(spec, blocks, flags=0):
    sink = G.CollectingSink()
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    with G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 100.0, 100.0, sink,
                             input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL, flags=flags) as gs:
        hdr = _header()
        gs.init(G.RawBytes(hdr))
        for b in blocks:
            gs(G.RawBytes(b))
        out_bytes = int(gs.info().output_bytes)
        n_out = int(gs.info().n_out)
    return sink, out_bytes, n_out


def _oracle_check(spec, blocks, g):
    cfg = oracle_config(spec, "intended")
    orc = O.OracleSpectrometer(cfg)
    refs = [p for p in (orc(b)[1] for b in blocks) if p is not None]
    n_out = cfg.n_out
    assert g.rows == len(refs) * n_out
    for i, ref in enumerate(refs):
        assert np.array_equal(g.n0[i * n_out:(i + 1) * n_out], ref["n0"])
        assert np.array_equal(g.n1[i * n_out:(i + 1) * n_out], ref["n1"])
        assert O.rel_err(g.spectra[i * n_out:(i + 1) * n_out], ref["spec"]) <= SPEC_TOL


@pytest.mark.parametrize("spec", CASES, ids=[c.name for c in CASES])
def test_cpp_ring_pipeline(tmp_path, spec):
    G.load_library()
    pkg = os.path.join(ROOT, "psrdada_cpp_gb300")
    exe = str(tmp_path / "ring_pipeline")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                        os.path.join(ROOT, "tests", "cpp", "ring_pipeline.cpp"), "-o", exe, "-L", pkg, "-lgspec",
                        "-Wl,-rpath," + pkg, "-lpthread"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    blocks = [synth.make_block(spec, seed=21, block_index=i, lost_frac=0.05) for i in range(7)]
    dada = tmp_path / "in.dada"
    dada.write_bytes(_header().tobytes() + b"".join(b.tobytes() for b in blocks))
    sink, out_bytes, _ = _direct(spec, blocks)
    outp = tmp_path / "out.dat"
    r = subprocess.run([exe, str(dada), str(outp), str(spec.buffer_size), str(spec.heap_size), "1",
                        str(spec.fft_length), str(spec.naccumulate), str(spec.nbits), "1" if spec.dual_pol else "0",
                        str(out_bytes)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr + r.stdout
    assert f"blocks {len(blocks)} outputs {len(sink.blocks)} page_locked 1" in r.stdout, r.stdout
    data = outp.read_bytes()
    assert data[:4096] == bytes(sink.header[:4096]).ljust(4096, b"\0")[:4096]
    assert data[4096:] == b"".join(x.tobytes() for x in sink.blocks)
    _oracle_check(spec, blocks, gated_file.read_gated_file(str(outp)))


@pytest.mark.parametrize("spec", CASES, ids=[c.name for c in CASES])
def test_python_ring_pipeline(spec):
    """Producer thread -> page-locked MemoryRing -> DadaInputStream ->
    GatedSpectrometer -> DadaOutputStream -> MemoryRing -> drain thread."""
    blocks = [synth.make_block(spec, seed=22, block_index=i, lost_frac=0.05) for i in range(6)]
    ref, out_bytes, _ = _direct(spec, blocks)
    rin = ring.MemoryRing(spec.buffer_size, 3, page_lock=True)
    rout = ring.MemoryRing(out_bytes, 2)
    assert rin.page_locked

    def produce():
        import ctypes
        w = rin.writer()
        h = w.header_stream().next()
        hdr = _header()
        ctypes.memmove(h.ptr(), hdr.ctypes.data, hdr.size)
        h.used_bytes(hdr.size)
        w.header_stream().release()
        for b in blocks:
            d = w.data_stream().next()
            ctypes.memmove(d.ptr(), b.ctypes.data, b.size)
            d.used_bytes(b.size)
            w.data_stream().release()
        w.data_stream().end_of_data()

    got = G.CollectingSink()
    drained = []
    t_in = threading.Thread(target=produce)
    t_out = threading.Thread(target=lambda: drained.append(ring.DadaInputStream(rout.reader(), got).start()))
    t_in.start()
    t_out.start()
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    with G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 100.0, 100.0,
                             ring.DadaOutputStream(rout.writer()),
                             input_type=G.DUAL_POL if spec.dual_pol else G.SINGLE_POL) as gs:
        n = ring.DadaInputStream(rin.reader(), gs).start()
    rout.writer().data_stream().end_of_data()
    t_in.join()
    t_out.join()
    rin.close()
    assert n == len(blocks) and drained == [len(ref.blocks)]
    assert got.header[:4096] == ref.header[:4096]
    assert len(got.blocks) == len(ref.blocks)
    for a, b in zip(got.blocks, ref.blocks):
        assert np.array_equal(a, b)


def test_gated_file_with_saturation_record(tmp_path):
    """Handler -> SimpleFileWriter with the saturation extension record ->
    gated-file reader: spectra, counters and saturation counts as the oracle."""
    spec = S("ring_sat", 12, True, 6144, 1, 1 << 15, 1024, 8, diode_period_heaps=2)
    blocks = [synth.make_block(spec, seed=23, block_index=i, kind="c3") for i in range(6)]
    path = str(tmp_path / "sat.dat")
    w = G.SimpleFileWriter(path)
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, spec.n_side_channels)
    with G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 100.0, 100.0, w,
                             input_type=G.DUAL_POL, flags=G.FLAG_SATURATION_RECORD) as gs:
        gs.init(G.RawBytes(_header()))
        for b in blocks:
            gs(G.RawBytes(b))
        n_out = int(gs.info().n_out)
    w.close()
    g = gated_file.read_gated_file(path, records_per_block=n_out, saturation_record=True)
    _oracle_check(spec, blocks, g)
    cfg = oracle_config(spec, "intended")
    orc = O.OracleSpectrometer(cfg)
    refs = [p for p in (orc(b)[1] for b in blocks) if p is not None]
    assert np.array_equal(g.saturation[:, 0], np.concatenate([r["sat0"] for r in refs]))
    assert np.array_equal(g.saturation[:, 1], np.concatenate([r["sat1"] for r in refs]))
    assert int(g.saturation.sum()) > 0
