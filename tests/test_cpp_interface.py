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


def test_cpp_fits_round_trip(tmp_path):
    """profit_cuda::from_fits / to_fits (no GPU): a reference-written FITS
    file read and written back gives the reference's bytes when the offset
    and scale are the ones it was written with (the scale read back is
    CDELT's six-decimal value, exact for these fixtures); a missing file
    raises invalid_file."""
    import json
    import __graft_entry__
    __graft_entry__.build_cuda()
    lib_dir = os.path.join(ROOT, "libprofit_gb300")
    exe = str(tmp_path / "fits_example")
    cmd = ["g++", "-std=c++11", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "fits_example.cpp"), "-o", exe,
           "-L" + lib_dir, "-lpfcuda", "-Wl,-rpath," + lib_dir]
    subprocess.run(cmd, check=True, capture_output=True, text=True)
    fits_dir = os.path.join(ROOT, "tests", "golden", "fits")
    meta = json.loads(str(np.load(os.path.join(fits_dir, "manifest.npz"))["meta"]))
    for name in ("ramp_7x5", "noise_13x11_offset", "moffat_psf_25", "block_aligned_40x36"):
        src = os.path.join(fits_dir, name + ".fits")
        ox, oy = meta[name]["offset"]
        r = subprocess.run([exe, src, str(tmp_path / name), str(ox), str(oy)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        assert open(src, "rb").read() == (tmp_path / (name + ".fits")).read_bytes(), name
    r = subprocess.run([exe, str(tmp_path / "missing.fits"), str(tmp_path / "x"), "0", "0"], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "invalid_file: Couldn't open" in r.stdout
