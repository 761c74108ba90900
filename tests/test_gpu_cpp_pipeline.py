"""The C++ drop-in template end to end: a DADA file through the C++
FileInputStream -> GatedSpectrometer<...> -> file sink program
(tests/cpp/compile_handler.cpp, linked against libgspec.so) gives the same
bytes as the Python API and matches the oracle."""
import os
import subprocess

import numpy as np
import pytest

from oracle import gspec_oracle as O
from psrdada_cpp_gb300 import synth
import psrdada_cpp_gb300 as G
from tests.gpu_helpers import oracle_config, SPEC_TOL

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("ref_types", [False, True], ids=["own_types", "reference_types"])
@pytest.mark.parametrize("dual", [False, True])
def test_cpp_file_pipeline(tmp_path, dual, ref_types):
    """ref_types: the same program built against the reference's RawBytes and
    key-constructed DadaBufferLayout (header-only stand-ins)."""
    G.load_library()
    pkg = os.path.join(ROOT, "psrdada_cpp_gb300")
    exe = str(tmp_path / "pipeline")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include")]
                       + (["-DUSE_REFERENCE_TYPES"] if ref_types else []) +
                       [os.path.join(ROOT, "tests", "cpp", "compile_handler.cpp"), "-o", exe,
                        "-L", pkg, "-lgspec", "-Wl,-rpath," + pkg], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    if dual:
        spec = synth.StreamSpec("cppd", 12, True, 6144, 1, 1 << 15, 1024, 8, diode_period_heaps=2)
    else:
        spec = synth.StreamSpec("cpps", 8, False, 4096, 1, 1 << 15, 512, 8, diode_period_heaps=2)
    blocks = [synth.make_block(spec, seed=9, block_index=i, lost_frac=0.05) for i in range(6)]
    header = bytearray(4096)
    header[:22] = b"HDR_VERSION 1.0\nNBIT 8\n"[:22]
    dada = tmp_path / "in.dada"
    with open(dada, "wb") as f:
        f.write(bytes(header))
        for b in blocks:
            f.write(b.tobytes())
    outp = tmp_path / "out.dat"
    r = subprocess.run([exe, str(dada), str(outp), str(spec.buffer_size), str(spec.heap_size), "1",
                        str(spec.fft_length), str(spec.naccumulate), str(spec.nbits), "1" if dual else "0"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr + r.stdout
    data = outp.read_bytes()
    hdr = data[:4096].split(b"\0")[0].decode()
    assert "fft_length               %d\n" % spec.fft_length in hdr
    body = data[4096:]
    # the Python API on the same blocks
    sink = G.CollectingSink()
    lay = G.DadaBufferLayout(spec.buffer_size, spec.heap_size, 1)
    with G.GatedSpectrometer(lay, 0, 0, spec.fft_length, spec.naccumulate, spec.nbits, 100.0, 100.0, sink,
                             input_type=G.DUAL_POL if dual else G.SINGLE_POL) as gs:
        for b in blocks:
            gs(G.RawBytes(b))
    assert body == b"".join(x.tobytes() for x in sink.blocks)
    # and the oracle
    cfg = oracle_config(spec, "intended")
    orc = O.OracleSpectrometer(cfg)
    refs = [p for p in (orc(b)[1] for b in blocks) if p is not None]
    assert len(body) == len(refs) * cfg.output_bytes
    for i, ref in enumerate(refs):
        chunk = body[i * cfg.output_bytes:(i + 1) * cfg.output_bytes]
        sf, n0, n1 = O.parse_output(chunk, cfg)
        assert np.array_equal(n0, ref["n0"]) and np.array_equal(n1, ref["n1"])
        assert O.rel_err(sf, ref["spec"]) <= SPEC_TOL
