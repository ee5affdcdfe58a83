"""Adjoint against central finite differences of the FP64 oracle (GPU).

chi^2 = sum ((model - data) / sigma)^2 over small two-component models (a
boxy sersic bulge and a sersic disk, convolved by a Moffat PSF, plus a sky);
data = the oracle's image at parameters perturbed by 5 %, plus noise. The
gradient with respect to all 17 parameters (8 per sersic, bg) must match
central differences of the oracle's chi^2 with h = 1e-6 relative, by the
criterion of tests/helpers.py:
  |g - fd| <= 1e-4 |fd| + 1e-14 sum|c m| / h
              (+ 2e-6 sum|c dm/dpar| + 2e-6 sum 2|m dm/dpar| / sigma^2 in FP32)
(the second term the differences' own rounding, the others the scale of the
sum an FP32 gradient is and its sensitivity to the FP32 image's relative
error; c = 2 (m - d) / sigma^2).
Parameters whose finite difference changes the oracle's subsampling tree
(level counts at +-h differ) are excluded, as the adjoint holds the tree
fixed; the test asserts that at least 15 of the 17 remain.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PSF_SIZE = 15
MAGZERO = 25.0


def _specs(rng):
    import workloads as W
    psf = W.moffat_psf(PSF_SIZE, 3.0, 2.5)
    base = [
        ("sersic", dict(xcen=31.3, ycen=29.6, mag=16.0, re=4.5, nser=3.3, ang=33.0, axrat=0.7, box=0.15,
                        convolve=True)),
        ("sersic", dict(xcen=32.8, ycen=30.9, mag=15.5, re=9.0, nser=1.1, ang=112.0, axrat=0.4, box=0.0,
                        convolve=True)),
        ("sky", dict(bg=1.0)),
    ]
    return psf, base


def _order(profiles):
    names = []
    for i, (kind, params) in enumerate(profiles):
        if kind == "sersic":
            for k in ("xcen", "ycen", "mag", "ang", "axrat", "box", "re", "nser"):
                names.append((i, k))
        elif kind == "sky":
            names.append((i, "bg"))
    return names


SLOT = {"xcen": 0, "ycen": 1, "mag": 2, "ang": 3, "axrat": 4, "box": 5, "re": 6, "nser": 7, "bg": 6}


def _with(profiles, i, k, v):
    from tests.helpers import with_param
    return with_param(profiles, i, k, v)


@pytest.fixture(scope="module")
def problem(oracle_lib):
    return make_problem(oracle_lib)


def make_problem(O):
    rng = np.random.default_rng(2024)
    psf, truth = _specs(rng)
    perturbed = []
    for kind, p in truth:
        q = dict(p)
        for k in q:
            if k not in ("convolve",):
                q[k] = q[k] * (1 + 0.05 * rng.normal()) if k not in ("xcen", "ycen") else q[k] + 0.3 * rng.normal()
        if kind == "sersic":
            q["axrat"] = min(q["axrat"], 1.0)
        perturbed.append((kind, q))
    data, _, _ = O.evaluate(O.Case(64, 64, truth, psf=psf, magzero=MAGZERO))
    sigma = 0.01 * data.max()
    data = data + rng.normal(0, sigma, data.shape)
    return psf, perturbed, data, np.full_like(data, sigma)


def _chi2(O, psf, profiles, data, sigma):
    img, _, counts = O.evaluate(O.Case(64, 64, profiles, psf=psf, magzero=MAGZERO))
    return float(np.sum(((img - data) / sigma) ** 2)), counts


def _fd(O, psf, profiles, data, sigma):
    from tests.helpers import fd_gradients

    def render(p):
        img, _, counts = O.evaluate(O.Case(64, 64, p, psf=psf, magzero=MAGZERO))
        return img, counts
    return fd_gradients(render, profiles, _order(profiles), data, sigma)[1]


@pytest.fixture(scope="module")
def fd(problem, oracle_lib):
    psf, profiles, data, sigma = problem
    return _fd(oracle_lib, psf, profiles, data, sigma)


def _gpu_grad(problem, use_double, convolver=None):
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    psf, profiles, data, sigma = problem
    env = pg.get_cuda_environment(0, use_double=use_double)
    m = W.to_model(dict(width=64, height=64, psf=psf, profiles=profiles, magzero=MAGZERO), env)
    if convolver:
        m.set_convolver(convolver)
    b = pg.Batch([m], env)
    b.enable_adjoint()
    dt = torch.float64 if use_double else torch.float32
    img = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
    d = torch.tensor(data.ravel(), dtype=dt, device="cuda")
    s = torch.tensor(sigma.ravel(), dtype=dt, device="cuda")
    chi2 = torch.zeros(1, dtype=torch.float64, device="cuda")
    grad = torch.zeros(len(profiles) * 12, dtype=torch.float64, device="cuda")
    b.forward_backward(img, d, s, chi2, grad)
    b.check()
    return chi2.item(), grad.cpu().numpy().reshape(len(profiles), 12)


@pytest.mark.parametrize("use_double,convolver", [(True, None), (False, None), (False, "fft")])
def test_gradient_matches_finite_differences(problem, fd, oracle_lib, use_double, convolver):
    psf, profiles, data, sigma = problem
    chi2, grad = _gpu_grad(problem, use_double, convolver)
    chi2_ref, _ = _chi2(oracle_lib, psf, profiles, data, sigma)
    assert abs(chi2 - chi2_ref) <= (1e-10 if use_double else 1e-5) * chi2_ref
    checked = 0
    for (i, k), r in fd.items():
        if not r.usable:
            continue
        r.check(grad[i, SLOT[k]], not use_double, "%s[%d]" % (k, i))
        checked += 1
    assert checked >= 15


def test_cotangent_vjp(problem, oracle_lib):
    """With a cotangent c, pf_backward returns d(sum c * image)/d par."""
    import torch
    import libprofit_gb300 as pg
    import workloads as W
    O = oracle_lib
    psf, profiles, data, sigma = problem
    rng = np.random.default_rng(5)
    cot = rng.normal(size=data.shape)
    env = pg.get_cuda_environment(0, use_double=True)
    m = W.to_model(dict(width=64, height=64, psf=psf, profiles=profiles, magzero=MAGZERO), env)
    b = pg.Batch([m], env)
    b.enable_adjoint()
    img = torch.zeros(b.total_pixels, dtype=torch.float64, device="cuda")
    b.forward(img)
    grad = torch.zeros(len(profiles) * 12, dtype=torch.float64, device="cuda")
    c = torch.tensor(cot.ravel(), dtype=torch.float64, device="cuda")
    b.backward(img, cotangent=c, grad=grad)
    b.check()
    g = grad.cpu().numpy().reshape(len(profiles), 12)
    for (i, k) in [(0, "re"), (1, "xcen"), (1, "nser"), (2, "bg")]:
        v = profiles[i][1][k]
        h = 1e-6 * max(abs(v), 1e-3)
        ip, _, _ = O.evaluate(O.Case(64, 64, _with(profiles, i, k, v + h), psf=psf, magzero=MAGZERO))
        im, _, _ = O.evaluate(O.Case(64, 64, _with(profiles, i, k, v - h), psf=psf, magzero=MAGZERO))
        want = float(np.sum(cot * (ip - im)) / (2 * h))
        assert abs(g[i, SLOT[k]] - want) <= 1e-4 * abs(want) + 1e-8, (k, g[i, SLOT[k]], want)


def test_fft_adjoint_matches_direct(problem):
    """FP32 path: the FFT convolution's adjoint (the cotangent correlated with
    the PSF through the spectrum) against the direct convolution's adjoint on
    the same model and data: chi^2 within 1e-6, every gradient within
    1e-4 relative (plus 1e-7 of the largest)."""
    chi2_d, g_d = _gpu_grad(problem, False, "brute")
    chi2_f, g_f = _gpu_grad(problem, False, "fft")
    assert abs(chi2_f - chi2_d) <= 1e-6 * chi2_d
    scale = np.abs(g_d).max()
    np.testing.assert_allclose(g_f, g_d, rtol=1e-4, atol=1e-7 * scale)
