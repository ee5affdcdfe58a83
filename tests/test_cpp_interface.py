"""The C++ host interface (include/profit_cuda.hpp) compiles against the C ABI
(CPU), and a libprofit-style program built on it reproduces the reference's
known answers and a golden image (GPU)."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "model_example.cpp")


def _compile(out):
    import __graft_entry__
    __graft_entry__.build_cuda()
    lib_dir = os.path.join(ROOT, "libprofit_gb300")
    cmd = ["g++", "-std=c++11", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), SRC, "-o", out,
           "-L" + lib_dir, "-lpfcuda", "-Wl,-rpath," + lib_dir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)


def test_cpp_interface_compiles(tmp_path):
    _compile(str(tmp_path / "model_example"))


@pytest.mark.gpu
def test_cpp_program_matches_reference(tmp_path):
    from tests.golden.load import load
    golden = load()["cfg1_sersic_brute"]
    exe = str(tmp_path / "model_example")
    _compile(exe)
    psf_path, out_path = str(tmp_path / "psf.bin"), str(tmp_path / "out.bin")
    np.ascontiguousarray(golden["psf"], dtype=np.float64).tofile(psf_path)
    r = subprocess.run([exe, psf_path, out_path], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "ok" in r.stdout
    img = np.fromfile(out_path, dtype=np.float64).reshape(100, 100)
    ref = golden["image"]
    assert np.max(np.abs(img - ref) / np.abs(ref)) <= 1e-10
