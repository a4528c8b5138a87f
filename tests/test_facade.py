"""The C++ facade include/lsgpu.hpp (reference class names and signatures over the C ABI): it
compiles and links against the library here; on a GPU its results equal the C ABI's bit for bit."""
import os
import subprocess

import pytest

from casl_p4est_gb300 import _lib as L

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_check(tmp_path):
    exe = str(tmp_path / "facade_check")
    lib_dir = os.path.dirname(L.LIB_PATH)
    subprocess.run(["g++", "-std=c++17", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "facade_check.cpp"), "-L", lib_dir, "-llsgpu",
                    "-Wl,-rpath," + lib_dir, "-o", exe], check=True)
    return exe


def test_facade_compiles_and_links(tmp_path):
    assert os.path.exists(build_check(tmp_path))


@pytest.mark.gpu
def test_facade_matches_c_abi(tmp_path):
    out = subprocess.run([build_check(tmp_path)], capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    assert "facade ok" in out.stdout
