"""The CUDA convolver bound to the reference library itself (CPU).

include/profit_cuda_convolver.hpp is a profit::Convolver for the unmodified
libprofit's Model::set_convolver. Where the reference's sources are present
(oracle/_ref holds them compiled, see oracle/Makefile), a program using the
reference's own Model with that convolver is compiled and linked against the
compiled reference and libpfcuda, and run without a GPU: the C ABI's failures
reach it as the reference's exceptions (invalid_parameter for an invalid
argument, a profit::exception for the missing device). Elsewhere the test is
skipped: the reference's headers are needed to compile the binding.
"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _reference_tree():
    d = os.environ.get("PF_REFERENCE_DIR")
    if not d:
        import __graft_entry__
        d = __graft_entry__.REFERENCE_TREE
    return d if os.path.isdir(os.path.join(d, "include", "profit")) else None


def build_example(out):
    ref = _reference_tree()
    ref_lib = os.path.join(ROOT, "oracle", "_ref")
    if ref is None or not os.path.exists(os.path.join(ref_lib, "libprofit_ref.so")):
        pytest.skip("the reference's headers and compiled library are not on this host")
    import __graft_entry__
    __graft_entry__.build_cuda()
    lib_dir = os.path.join(ROOT, "libprofit_gb300")
    cmd = ["g++", "-std=c++11", "-O2", "-Wall", "-I" + os.path.join(ref_lib, "include"),
           "-I" + os.path.join(ref, "include"), "-I" + os.path.join(ROOT, "include"),
           os.path.join(ROOT, "tests", "cpp", "ref_convolver_example.cpp"), "-o", out,
           "-L" + ref_lib, "-lprofit_ref", "-L" + lib_dir, "-lpfcuda",
           "-Wl,-rpath," + ref_lib, "-Wl,-rpath," + lib_dir]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_reference_model_with_cuda_convolver_errors(tmp_path):
    exe = str(tmp_path / "ref_convolver_example")
    build_example(exe)
    r = subprocess.run([exe, "errors"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "invalid_parameter: pf_convolve: NULL argument" in r.stdout
    assert "errors ok" in r.stdout
