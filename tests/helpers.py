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


# ---------------------------------------------------------------- gradients
#
# The adjoint is checked against central differences of the FP64 oracle's
# chi^2 = sum ((m - d) / sigma)^2, step h = FD_STEP x |parameter|. A gradient
# g passes when
#   |g - fd| <= GRAD_RTOL |fd| + noise
#               (+ FP32_COND x cond + FP32_IMAGE x sens for FP32 results)
# where
#   noise = FD_NOISE x sum_p |c_p m_p| / h, c = 2 (m - d) / sigma^2: the
#           rounding of the two chi^2 values the difference divides by 2h
#           (their pixels carry ~1e-16 relative rounding; measured on these
#           problems as ~1.1e-16 x sum |c m| / h, the floor is ~100 times
#           that);
#   cond  = sum_p |c_p dm_p / dtheta| (dm/dtheta from the same differences):
#           the scale of the sum the gradient is. An FP32 result carries
#           rounding of a few units of 2^-24 on that scale, whatever the
#           gradient's own size; a component that nearly cancels (|g| much
#           smaller than cond) can hold no more relative precision than that;
#   sens  = sum_p 2 |m_p dm_p / dtheta| / sigma_p^2: the gradient's
#           sensitivity to relative errors of the image m, which an FP32
#           image carries at ~1e-7 (a few 1e-6 at most, on faint pixels).
# Parameters whose +-h changes the oracle's subsampling tree (per-level
# counts) are not checked: the adjoint holds the tree fixed.
FD_STEP = 1e-6
FD_NOISE = 1e-14
FP32_COND = 2e-6
FP32_IMAGE = 2e-6
GRAD_RTOL = 1e-4


class FD:
    """One parameter's central difference and the floors of its check."""

    def __init__(self, fd, usable, h, noise, cond, sens):
        self.fd, self.usable, self.h, self.noise, self.cond, self.sens = fd, usable, h, noise, cond, sens

    def bound(self, single):
        fp32 = FP32_COND * self.cond + FP32_IMAGE * self.sens if single else 0.0
        return GRAD_RTOL * abs(self.fd) + self.noise + fp32

    def check(self, got, single, what=""):
        err = abs(got - self.fd)
        assert err <= self.bound(single), "%s: adjoint %.10g vs fd %.10g (err %.3g, 1e-4|fd| %.3g, noise %.3g, " \
            "cond %.3g, sens %.3g)" % (what, got, self.fd, err, GRAD_RTOL * abs(self.fd), self.noise, self.cond,
                                       self.sens)


def fd_gradients(render, profiles, names, data, sigma, smooth=False):
    """Central differences of chi^2 for the parameters `names` ((profile
    index, parameter name) pairs). render(profiles) -> (image, level counts)
    from the FP64 oracle. With smooth=True a parameter is also unusable when
    its quotient moves by more than 2e-5 relative (plus ten times the noise)
    at h / 10: a sub-point near a cusp makes the difference depart from the
    derivative. Returns (chi^2, {(i, name): FD})."""
    img0, counts0 = render(profiles)
    cot = 2 * (img0 - data) / sigma ** 2
    chi0 = float(np.sum(((img0 - data) / sigma) ** 2))
    scale = float(np.sum(np.abs(cot * img0)))
    msens = 2 * np.abs(img0) / sigma ** 2

    def chi(img):
        return float(np.sum(((img - data) / sigma) ** 2))

    out = {}
    for i, k in names:
        v = profiles[i][1][k]
        h = FD_STEP * max(abs(v), 1e-3)
        ip, cp = render(with_param(profiles, i, k, v + h))
        im, cm = render(with_param(profiles, i, k, v - h))
        fd = (chi(ip) - chi(im)) / (2 * h)
        dm = np.abs(ip - im) / (2 * h)
        cond = float(np.sum(np.abs(cot) * dm))
        sens = float(np.sum(msens * dm))
        usable = np.array_equal(cp, counts0) and np.array_equal(cm, counts0)
        noise = FD_NOISE * scale / h
        if smooth and usable:
            ip2, _ = render(with_param(profiles, i, k, v + h / 10))
            im2, _ = render(with_param(profiles, i, k, v - h / 10))
            fd2 = (chi(ip2) - chi(im2)) / (2 * h / 10)
            usable = abs(fd - fd2) <= 2e-5 * abs(fd) + 10 * noise
        out[(i, k)] = FD(fd, usable, h, noise, cond, sens)
    return chi0, out


def with_param(profiles, i, k, v):
    """A copy of `profiles` ((kind, params) pairs) with profile i's k set to v."""
    out = [(kind, dict(p)) for kind, p in profiles]
    out[i][1][k] = v
    return out
