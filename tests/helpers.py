"""Shared test helpers: build product models from the golden case specs."""
import numpy as np

import libprofit_gb300 as pg


def product_model(spec, psf, env=None):
    """A libprofit_gb300.Model equivalent to a tests/golden/cases.py spec."""
    m = pg.Model(spec["width"], spec["height"])
    m.set_image_pixel_scale(spec.get("scale", (1.0, 1.0)))
    m.set_magzero(spec.get("magzero", 0.0))
    m.set_finesampling(spec.get("finesampling", 1))
    m.set_return_finesampled(spec.get("return_finesampled", True))
    if psf is not None:
        m.set_psf(psf)
    if spec.get("mask") is not None:
        m.set_mask(np.asarray(spec["mask"], dtype=np.uint8))
        m.set_adjust_mask(spec.get("adjust_mask", True))
    if env is not None:
        m.set_cuda_env(env)
    for kind, params in spec["profiles"]:
        p = m.add_profile(kind)
        for k, v in params.items():
            if k in ("convolve", "rough", "adjust", "rescale_flux"):
                p.parameter(k, bool(v))
            elif k in ("resolution", "max_recursions"):
                p.parameter(k, int(v))
            else:
                p.parameter(k, float(v))
    return m


def rel_err(a, b, floor=0.0):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    den = np.maximum(np.abs(b), floor)
    with np.errstate(invalid="ignore", divide="ignore"):
        r = np.where(den > 0, np.abs(a - b) / np.where(den > 0, den, 1), np.abs(a - b))
    return float(np.nanmax(r)) if r.size else 0.0
