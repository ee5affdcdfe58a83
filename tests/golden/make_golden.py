"""Generates tests/golden/reference_images.npz from the UNMODIFIED libprofit.

Run from the repository root where the reference tree exists:
    python tests/golden/make_golden.py
It builds oracle/_ref/libprofit_ref.so (oracle/Makefile, target `ref`),
evaluates every case of tests/golden/cases.py through the reference's public
C++ API (profit::Model, add_profile, parameter, set_psf, create_convolver,
Model::evaluate) and stores, per case, the output image and the per-level
subsampling counts (PROFIT_DEBUG's n_integrations, one radial profile per
case). PSFs named by another case are that case's rendered image, normalised
by Model::set_psf.
"""
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from tests.golden.cases import golden_cases, resolve_psf  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_images.npz")


def to_case(spec, psf):
    return O.Case(spec["width"], spec["height"], spec["profiles"], psf=psf,
                  scale=spec.get("scale", (1.0, 1.0)), magzero=spec.get("magzero", 0.0),
                  finesampling=spec.get("finesampling", 1),
                  return_finesampled=spec.get("return_finesampled", True),
                  convolver=spec.get("convolver", "brute"),
                  mask=None if spec.get("mask") is None else np.asarray(spec["mask"], dtype=np.uint8),
                  adjust_mask=spec.get("adjust_mask", True))


def main():
    O.build(with_ref=True)
    cases = golden_cases()
    rendered = {}
    arrays = {}
    meta = {}
    for name, spec in cases.items():
        psf = resolve_psf(spec, rendered)
        img, counts = O.evaluate_reference(to_case(spec, psf), threads=1)
        rendered[name] = img
        arrays["img__" + name] = img
        arrays["cnt__" + name] = counts
        meta[name] = {"shape": list(img.shape)}
    arrays["meta"] = np.frombuffer(json.dumps(meta, sort_keys=True).encode(), dtype=np.uint8)
    np.savez_compressed(OUT, **arrays)
    print("wrote", OUT, len(cases), "cases")


if __name__ == "__main__":
    main()
