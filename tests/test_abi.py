"""The C-ABI library: builds, loads without a GPU, exports every entry point
include/gspec.h declares, validates configurations before touching CUDA, and
the Python mirror fails loudly without it (no CPU fallback)."""
import ctypes
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER_DIR = os.path.join(ROOT, "include")


def _lib_path():
    from psrdada_cpp_gb300.gated_spectrometer import LIB_PATH
    if not LIB_PATH.exists():
        from psrdada_cpp_gb300.build import build
        build()
    return str(LIB_PATH)


def declared_symbols():
    names = set()
    for fn in os.listdir(HEADER_DIR):
        if fn.endswith(".h"):
            text = open(os.path.join(HEADER_DIR, fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(gspec_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_every_declared_symbol_is_exported():
    lib = ctypes.CDLL(_lib_path())
    syms = declared_symbols()
    assert "gspec_create" in syms and "gspec_process" in syms and "gspec_init" in syms
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing


def test_configuration_errors_without_gpu():
    from psrdada_cpp_gb300.gated_spectrometer import GspecConfig, load_library
    lib = load_library()
    err = ctypes.create_string_buffer(256)

    def create(**kw):
        base = dict(buffer_size=16 * 4104, heap_size=4096, n_side_channels=1, fft_length=1024, naccumulate=4,
                    nbits=8)
        base.update(kw)
        h = lib.gspec_create(ctypes.byref(GspecConfig(**base)), err, 256)
        if h:                      # only a valid configuration on a machine with a GPU
            lib.gspec_destroy(h)
            return None
        return err.value.decode()

    assert "nbits" in create(nbits=16)
    assert "power of two" in create(fft_length=1000)
    assert "not implemented" in create(input_type=1, output_type=0)
    assert "multiple" in create(naccumulate=3)
    assert "selected_side_channel" in create(selected_side_channel=2)
    assert "tile" in create(convention=1, heap_size=8192, buffer_size=16 * 8200)
    # a valid configuration fails only where CUDA starts (on a machine without a GPU)
    msg = create()
    assert msg is None or "cudaSetDevice" in msg or "CUDA" in msg or msg == ""


def test_misaligned_device_pointers_are_rejected_before_cuda():
    """An unaligned block or output pointer is an argument error, found on the
    host before any CUDA call (so no kernel ever reads it)."""
    from psrdada_cpp_gb300.gated_spectrometer import GspecConfig, load_library
    lib = load_library()
    err = ctypes.create_string_buffer(256)
    cfg = GspecConfig(buffer_size=16 * 4104, heap_size=4096, n_side_channels=1, fft_length=1024, naccumulate=4,
                      nbits=8)
    fn = lib.gspec_process_block_noalloc
    fn.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                   ctypes.c_char_p, ctypes.c_size_t]
    aligned, odd = 1 << 20, (1 << 20) + 8
    for blk, out in ((odd, aligned), (aligned, odd)):
        rc = fn(ctypes.byref(cfg), blk, aligned, out, None, err, 256)
        assert rc == -1 and b"aligned" in err.value, (rc, err.value)
    assert lib.gspec_run_block_device(None, aligned, aligned, None) == -1   # null handle


def test_python_mirror_fails_loudly_without_library(tmp_path):
    code = (
        "import psrdada_cpp_gb300.gated_spectrometer as g, pathlib;"
        "g.LIB_PATH = pathlib.Path('%s');"
        "g._LIB = None\n"
        "try:\n"
        "    g.GatedSpectrometer(g.DadaBufferLayout(16*4104, 4096, 1), 0, 0, 1024, 4, 8, 1.0, 1.0, g.NullSink())\n"
        "except RuntimeError as e:\n"
        "    print('RAISED', e)\n" % (tmp_path / "missing.so"))
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True)
    assert "RAISED" in out.stdout and "missing" in out.stdout


def test_cpp_header_compiles():
    """The C++ drop-in template (include/psrdada_cpp_gb300/GatedSpectrometer.hpp)
    compiles against a NullSink-style handler with plain g++."""
    src = os.path.join(ROOT, "tests", "cpp", "compile_handler.cpp")
    if not os.path.exists(src):
        pytest.skip("no C++ compile probe")
    out = os.path.join(ROOT, "psrdada_cpp_gb300", "_build", "compile_handler.o")
    os.makedirs(os.path.dirname(out), exist_ok=True)
    r = subprocess.run(["g++", "-std=c++17", "-c", "-I", HEADER_DIR, src, "-o", out], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
