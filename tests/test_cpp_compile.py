"""The C++ drop-in header compiles against both the stand-alone types and the
reference's own RawBytes / key-constructed DadaBufferLayout (header-only
stand-ins with the reference's signatures): no GPU needed."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.parametrize("defines", [[], ["-DUSE_REFERENCE_TYPES"]], ids=["own_types", "reference_types"])
def test_drop_in_compiles(defines):
    if not shutil.which("g++"):
        pytest.skip("no g++")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Werror", "-I",
                        os.path.join(ROOT, "include"), "-I", os.path.join(ROOT, "tests", "cpp")] + defines +
                       [os.path.join(ROOT, "tests", "cpp", "compile_handler.cpp")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
