"""Loads tests/golden/reference_images.npz (made by make_golden.py from the
unmodified reference) and rebuilds each case as an oracle.Case."""
import json
import os

import numpy as np

from tests.golden.cases import golden_cases, resolve_psf

PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_images.npz")


def load():
    data = np.load(PATH)
    meta = json.loads(bytes(data["meta"]).decode())
    specs = golden_cases()
    rendered = {}
    out = {}
    for name, spec in specs.items():
        assert name in meta, name
        img = data["img__" + name]
        rendered[name] = img
        out[name] = dict(spec=spec, psf=resolve_psf(spec, rendered), image=img,
                         counts=data["cnt__" + name])
    return out


def to_case(O, entry):
    spec = entry["spec"]
    return O.Case(spec["width"], spec["height"], spec["profiles"], psf=entry["psf"],
                  scale=spec.get("scale", (1.0, 1.0)), magzero=spec.get("magzero", 0.0),
                  finesampling=spec.get("finesampling", 1),
                  return_finesampled=spec.get("return_finesampled", True),
                  convolver=spec.get("convolver", "brute"),
                  mask=None if spec.get("mask") is None else np.asarray(spec["mask"], dtype=np.uint8),
                  adjust_mask=spec.get("adjust_mask", True))
