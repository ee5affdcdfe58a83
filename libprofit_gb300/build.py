"""Builds libprofit_gb300/libpfcuda.so: the CUDA kernels and the C ABI of
include/pf_cuda.h, for sm_103a only.

Each translation unit is compiled in parallel with nvcc; the ones that must
round alike wherever they are inlined (the reference's FP64 arithmetic, the
single-precision evaluation) get -fmad=false.
Objects go to libprofit_gb300/_build/, the library next to this file. The
build is skipped when the library is newer than every source.
"""
import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpfcuda.so")
CLI_SRC = os.path.join(HERE, "cli", "profit_cli.cpp")
CLI = os.path.join(HERE, "profit-cli")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-I" + os.path.join(ROOT, "include")]
# translation units built without the compiler's multiply-add contraction:
# the two that reproduce the reference's double-precision arithmetic, and the
# single-precision evaluation, whose multiply-adds are explicit fmaf calls so
# that every kernel instance rounds alike (its FP64 re-takes then round as the
# double-precision path does)
NO_FMAD = {"setup.cu", "eval_f64.cu", "eval_f32.cu"}


def nvcc():
    path = shutil.which("nvcc")
    if path:
        return path
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpfcuda.so")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _deps():
    out = []
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            if f.endswith((".cu", ".cuh", ".h")):
                out.append(os.path.join(d, f))
    out.append(os.path.abspath(__file__))
    return out


def up_to_date(lib=LIB, user_profile=None):
    if not os.path.exists(lib):
        return False
    t = os.path.getmtime(lib)
    deps = _deps() + ([user_profile] if user_profile else [])
    return all(os.path.getmtime(p) <= t for p in deps)


def _compile(src, extra, build_dir=BUILD):
    obj = os.path.join(build_dir, src[:-3] + ".o")
    cmd = [nvcc()] + ARCH + COMMON + extra
    if src in NO_FMAD:
        cmd += ["-fmad=false"]
    cmd += ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj, r.stderr


def build_cli():
    """profit-cli for this backend (cli/profit_cli.cpp on include/profit_cuda.hpp),
    next to the library."""
    if os.path.exists(CLI) and os.path.getmtime(CLI) >= max(
            os.path.getmtime(p) for p in (LIB, CLI_SRC, os.path.join(ROOT, "include", "profit_cuda.hpp"))):
        return CLI
    cmd = [os.environ.get("CXX", "g++"), "-std=c++11", "-O2", "-Wall", "-I" + os.path.join(ROOT, "include"), CLI_SRC,
           "-o", CLI + ".tmp", "-L" + HERE, "-lpfcuda", "-Wl,-rpath,$ORIGIN"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("profit-cli build failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(CLI + ".tmp", CLI)
    return CLI


def build(force=False, verbose=False, extra=None, user_profile=None, out_dir=None):
    """Compiles every CUDA translation unit for sm_103a and links the library
    (and profit-cli on it). user_profile: a user-defined radial profile file
    to compile in (csrc/user_profile.cuh), out_dir: where that library goes
    (its own directory: libpfcuda.so and _build/), instead of next to this
    file."""
    lib, build_dir = LIB, BUILD
    if out_dir:
        lib, build_dir = os.path.join(out_dir, "libpfcuda.so"), os.path.join(out_dir, "_build")
    if user_profile:
        user_profile = os.path.abspath(user_profile)
        if not os.path.exists(user_profile):
            raise RuntimeError("user profile file not found: %s" % user_profile)
    if not force and up_to_date(lib, user_profile):
        if lib == LIB:
            build_cli()
        return lib
    os.makedirs(build_dir, exist_ok=True)
    extra = list(extra or [])
    if user_profile:
        extra.append('-DPF_USER_PROFILE_FILE="%s"' % user_profile)
    srcs = sources()
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        results = list(ex.map(lambda s: _compile(s, extra, build_dir), srcs))
    objs = [o for o, _ in results]
    if verbose:
        for _, err in results:
            if err.strip():
                sys.stderr.write(err)
    tmp = lib + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcudart_static"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    os.replace(tmp, lib)
    if lib == LIB:
        build_cli()
    return lib


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="builds libpfcuda.so (sm_103a) and profit-cli")
    ap.add_argument("--force", action="store_true")
    ap.add_argument("--ptxas", action="store_true", help="print ptxas register and spill figures")
    ap.add_argument("--user-profile", help="a user-defined radial profile file to compile in")
    ap.add_argument("--out", help="directory of the library built (default: next to this file)")
    a = ap.parse_args()
    print(build(force=a.force, verbose=True, extra=["-Xptxas", "-v"] if a.ptxas else None,
                user_profile=a.user_profile, out_dir=a.out))
