"""Generates the FITS fixtures under tests/golden/fits/ with the UNMODIFIED
libprofit (profit::to_fits, profit::from_fits; src/fits_utils.cpp).

Run from the repository root where the reference tree exists:
    python tests/golden/make_fits_golden.py
It builds oracle/_ref/libprofit_ref.so (oracle/Makefile, target `ref`) and,
for every case below, writes the image with the reference's to_fits into
tests/golden/fits/<name>.fits and reads it back with the reference's
from_fits. tests/golden/fits/manifest.npz keeps each case's input image,
offset and pixel scale, the image and scale from_fits returned, and the
reference's messages for the failure cases (files named relative to the
working directory, so that no path of this machine is recorded).
"""
import json
import os
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
import workloads as W  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "fits")


def cases():
    rng = np.random.Generator(np.random.PCG64(2880))
    specials = np.array([[0.0, -0.0, 5e-324], [1.7976931348623157e308, np.inf, -np.inf]])
    return {
        # name: (image, offset (whole pixels: the reference's Point), pixel scale)
        "ramp_7x5": (np.arange(35, dtype=np.float64).reshape(5, 7) * 0.25 - 3.0, (0, 0), (1.0, 1.0)),
        "noise_13x11_offset": (rng.standard_normal((11, 13)), (3, 17), (0.5, 0.2)),
        # 40 x 36 x 8 bytes = four whole blocks: a whole block of padding follows
        "block_aligned_40x36": (rng.uniform(-1, 1, (36, 40)), (0, 0), (2.0, 2.0)),
        "specials_3x2": (specials, (1, 0), (1.0, 1.0)),
        "moffat_psf_25": (W.moffat_psf(25, 3.0, 2.5), (12, 12), (0.2, 0.2)),
        # CDELT is written with six decimals: from_fits returns the rounded scale
        "long_scale_9x4": (rng.uniform(0, 10, (4, 9)), (0, 7), (0.123456789, 3.14159265)),
        "single_1x1": (np.array([[42.0]]), (0, 0), (1.0, 1.0)),
    }


def failure_messages(workdir):
    """The reference's messages for a missing file, a file that ends inside
    the header, and one whose data are shorter than NAXIS1 x NAXIS2."""
    cwd = os.getcwd()
    os.chdir(workdir)
    try:
        out = {}
        try:
            O.ref_from_fits("missing.fits")
        except O.OracleError as e:
            out["missing.fits"] = str(e)
        with open("header_cut.fits", "wb") as f:
            f.write(b"SIMPLE  =                    T".ljust(80) + b"NAXIS1  = 4".ljust(40))
        try:
            O.ref_from_fits("header_cut.fits")
        except O.OracleError as e:
            out["header_cut.fits"] = str(e)
        O.ref_to_fits(np.ones((4, 4)), (0, 0), (1, 1), "short_data.fits")
        data = open("short_data.fits", "rb").read()
        with open("short_data.fits", "wb") as f:
            f.write(data[:2880 + 100])  # the header and 100 of the 128 data bytes
        try:
            O.ref_from_fits("short_data.fits")
        except O.OracleError as e:
            out["short_data.fits"] = str(e)
        return out
    finally:
        os.chdir(cwd)


def main():
    O.build(with_ref=True)
    os.makedirs(OUT, exist_ok=True)
    arrays = {}
    meta = {}
    for name, (img, offset, scale) in cases().items():
        path = os.path.join(OUT, name + ".fits")
        O.ref_to_fits(img, offset, scale, path)
        back, back_scale = O.ref_from_fits(path)
        arrays["image_" + name] = img
        arrays["read_" + name] = back
        meta[name] = {"offset": list(offset), "scale": list(scale), "read_scale": list(back_scale),
                      "bytes": os.path.getsize(path)}
    with tempfile.TemporaryDirectory() as d:
        meta["_failures"] = failure_messages(d)
    np.savez_compressed(os.path.join(OUT, "manifest.npz"), meta=json.dumps(meta, sort_keys=True), **arrays)
    print(json.dumps(meta, indent=1, sort_keys=True))


if __name__ == "__main__":
    main()
