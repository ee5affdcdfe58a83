"""Calculation masks on the GPU paths (Model::set_mask, src/model.cpp:152-317).

The masked golden cases (rendered by the unmodified libprofit) run through
the generic golden tests of the FP64, FP32 and FFT paths; this file adds:
  * a batch mixing masked and unmasked models renders every model exactly as
    it renders alone (FP64, bit for bit) and as the reference did;
  * a mask used as given (set_adjust_mask(False): drawing dimensions, no
    padding logic, no final masking) against the oracle: FP64 <= 1e-10
    relative per pixel, FP32 at the single-precision bars;
  * the adjoint of chi^2 with a mask against central finite differences of
    the oracle (h = 1e-6 relative) with the bars of the unmasked adjoint test,
    for the FP64 path and the FP32 path with direct and FFT convolution;
  * pixels outside the mask are exactly 0 on every path.
"""
import numpy as np
import pytest

from tests.golden.load import load
from tests.helpers import product_model
from tests.test_gpu_adjoint import MAGZERO, SLOT, _order, _specs, _with

pytestmark = pytest.mark.gpu

GOLDEN = load()
MASKED = sorted(n for n in GOLDEN if GOLDEN[n]["spec"].get("mask") is not None)
SIDE = 64


@pytest.fixture(scope="module")
def envs():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    return pg.get_cuda_environment(0, use_double=True), pg.get_cuda_environment(0, use_double=False)


def test_masked_cases_present():
    assert len(MASKED) >= 7


def test_batch_mixes_masked_and_unmasked(envs):
    import torch
    import libprofit_gb300 as pg
    env64, _ = envs
    names = MASKED + ["cfg1_sersic_brute", "mixed_conv_sky_psf", "finesampled_downsampled"]
    models = [product_model(GOLDEN[n]["spec"], GOLDEN[n]["psf"], env64) for n in names]
    b = pg.Batch(models, env64)
    out = torch.zeros(b.total_pixels, dtype=torch.float64, device="cuda")
    b.forward(out)
    b.check()
    o = out.cpu().numpy()
    for i, n in enumerate(names):
        w, h = b.dims[i]
        img = o[b.offsets[i]:b.offsets[i + 1]].reshape(h, w)
        assert np.array_equal(img, models[i].evaluate()), n
        ref = GOLDEN[n]["image"]
        zero = ref == 0
        assert np.array_equal(img[zero], ref[zero]), n
        nz = ~zero
        assert not nz.any() or np.max(np.abs(img[nz] - ref[nz]) / np.abs(ref[nz])) <= 1e-10, n


def _given_mask_spec():
    """A 60 x 50 model, 15 x 15 PSF: drawing area 74 x 64 (half the PSF on
    each side); the mask covers that area directly."""
    import workloads as W
    rng = np.random.default_rng(77)
    psf = W.moffat_psf(15, 3.0, 2.5)
    mask = np.zeros((64, 74), np.uint8)
    mask[10:50, 12:60] = 1
    mask &= (rng.random(mask.shape) < 0.85).astype(np.uint8)
    profiles = [("sersic", dict(xcen=31.2, ycen=24.6, mag=15.0, re=6.0, nser=2.5, ang=40.0, axrat=0.6,
                                box=0.1, convolve=True)),
                ("sky", dict(bg=0.01))]
    return dict(width=60, height=50, psf=psf, mask=mask, adjust_mask=False, profiles=profiles)


@pytest.mark.parametrize("use_double", [True, False])
def test_mask_used_as_given(envs, oracle_lib, use_double):
    import workloads as W
    spec = _given_mask_spec()
    env = envs[0] if use_double else envs[1]
    img = W.to_model(spec, env).evaluate()
    ref, _, _ = oracle_lib.evaluate(W.to_oracle_case(spec))
    assert img.shape == ref.shape
    zero = ref == 0
    assert np.all(img[zero] == 0)
    nz = ~zero
    rel = np.abs(img[nz] - ref[nz]) / np.abs(ref[nz])
    if use_double:
        assert rel.max() <= 1e-10, rel.max()
    else:
        peak = np.abs(ref).max()
        bright = np.abs(ref) > 1e-9 * peak
        r = np.abs(img[bright] - ref[bright]) / np.abs(ref[bright])
        assert r.max() <= 1e-4, r.max()
        assert abs(img.sum() - ref.sum()) <= 1e-5 * abs(ref.sum())


def _fit_mask():
    """Pixels within an ellipse around the galaxy, with random holes."""
    rng = np.random.default_rng(9)
    y, x = np.mgrid[0:SIDE, 0:SIDE] + 0.5
    inside = ((x - 32) / 22.0) ** 2 + ((y - 30) / 16.0) ** 2 <= 1
    return (inside & (rng.random((SIDE, SIDE)) < 0.9)).astype(np.uint8)


@pytest.fixture(scope="module")
def masked_problem(oracle_lib):
    O = oracle_lib
    rng = np.random.default_rng(2025)
    psf, truth = _specs(rng)
    mask = _fit_mask()
    perturbed = []
    for kind, p in truth:
        q = dict(p)
        for k in q:
            if k != "convolve":
                q[k] = q[k] * (1 + 0.05 * rng.normal()) if k not in ("xcen", "ycen") else q[k] + 0.3 * rng.normal()
        if kind == "sersic":
            q["axrat"] = min(q["axrat"], 1.0)
        perturbed.append((kind, q))
    data, _, _ = O.evaluate(O.Case(SIDE, SIDE, truth, psf=psf, magzero=MAGZERO, mask=mask))
    sigma = 0.01 * data.max()
    data = data + rng.normal(0, sigma, data.shape)
    return psf, perturbed, mask, data, np.full_like(data, sigma)


def _chi2(O, psf, profiles, mask, data, sigma):
    img, _, counts = O.evaluate(O.Case(SIDE, SIDE, profiles, psf=psf, magzero=MAGZERO, mask=mask))
    return float(np.sum(((img - data) / sigma) ** 2)), counts, img


@pytest.fixture(scope="module")
def masked_fd(masked_problem, oracle_lib):
    psf, profiles, mask, data, sigma = masked_problem
    O = oracle_lib
    _, counts0, _ = _chi2(O, psf, profiles, mask, data, sigma)
    out = {}
    for i, k in _order(profiles):
        v = profiles[i][1][k]
        h = 1e-6 * max(abs(v), 1e-3)
        cp, c_p, _ = _chi2(O, psf, _with(profiles, i, k, v + h), mask, data, sigma)
        cm, c_m, _ = _chi2(O, psf, _with(profiles, i, k, v - h), mask, data, sigma)
        same_tree = np.array_equal(c_p, counts0) and np.array_equal(c_m, counts0)
        out[(i, k)] = ((cp - cm) / (2 * h), same_tree, h)
    return out


@pytest.mark.parametrize("use_double,convolver", [(True, None), (False, "brute"), (False, "fft")])
def test_masked_gradient_matches_finite_differences(envs, masked_problem, masked_fd, oracle_lib, use_double,
                                                    convolver):
    import torch
    import libprofit_gb300 as pg
    import workloads as W
    psf, profiles, mask, data, sigma = masked_problem
    env = envs[0] if use_double else envs[1]
    m = W.to_model(dict(width=SIDE, height=SIDE, psf=psf, profiles=profiles, magzero=MAGZERO, mask=mask), env)
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
    image = img.cpu().numpy().reshape(SIDE, SIDE)
    assert np.all(image[mask == 0] == 0), "pixels outside the mask must be 0"
    chi2_ref, _, _ = _chi2(oracle_lib, psf, profiles, mask, data, sigma)
    assert abs(chi2.item() - chi2_ref) <= (1e-10 if use_double else 1e-4) * chi2_ref
    g = grad.cpu().numpy().reshape(len(profiles), 12)
    rtol, floor = (1e-4, 1e-9) if use_double else (1e-3, 1e-6)
    checked = 0
    for (i, k), (want, same_tree, h) in masked_fd.items():
        if not same_tree:
            continue
        got = g[i, SLOT[k]]
        atol = floor * chi2_ref / h
        assert abs(got - want) <= rtol * abs(want) + atol, "%s[%d]: adjoint %.8g vs fd %.8g" % (k, i, got, want)
        checked += 1
    assert checked >= 15


# (model side, mask side, PSF side) of the reference's flux-capturing cases
# (tests/test_model.h:445-553): a sky of bg 1, optionally convolved with a
# uniform PSF, downsampled from finesampling 1 or 2, must give the unmasked
# image under the mask (1e-4 relative, exactly 0 elsewhere) for every
# placement of a square mask; all placements of one case run as one batch.
FLUX_CASES = [(20, 0, 5), (5, 2, 5), (5, 3, 5), (5, 4, 5), (5, 3, 4), (5, 4, 4), (5, 5, 4), (3, 1, 2),
              (20, 4, 5), (20, 5, 5), (20, 6, 5), (20, 5, 6), (20, 6, 6), (20, 7, 6), (20, 5, 9), (20, 5, 20),
              (20, 5, 30)]


def _sky_model(env, side, psf_side, convolver, fs, mask=None):
    import libprofit_gb300 as pg
    m = pg.Model(side, side)
    m.set_finesampling(fs)
    m.set_return_finesampled(False)
    m.set_psf(np.ones((psf_side, psf_side)))
    if convolver:
        m.set_convolver(convolver)
    m.set_cuda_env(env)
    p = m.add_profile("sky")
    p.parameter("bg", 1.0)
    if convolver:
        p.parameter("convolve", True)
    if mask is not None:
        m.set_mask(mask)
    return m


@pytest.mark.parametrize("case", FLUX_CASES, ids=lambda c: "%dx%d_mask%d_psf%d" % (c[0], c[0], c[1], c[2]))
def test_flux_captured_under_every_mask_placement(envs, case):
    import torch
    import libprofit_gb300 as pg
    side, mside, pside = case
    for use_double in (True, False):
        env = envs[0] if use_double else envs[1]
        dt = torch.float64 if use_double else torch.float32
        for convolver in (None, "brute", "fft"):
            for fs in (1, 2):
                full = _sky_model(env, side, pside, convolver, fs).evaluate()
                masks, models = [], []
                for oy in range(side - mside + 1):
                    for ox in range(side - mside + 1):
                        mk = np.zeros((side, side), np.uint8)
                        mk[oy:oy + mside, ox:ox + mside] = 1
                        masks.append(mk)
                        models.append(_sky_model(env, side, pside, convolver, fs, mk))
                b = pg.Batch(models, env)
                out = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
                b.forward(out)
                b.check()
                o = out.cpu().numpy().astype(np.float64)
                for i, mk in enumerate(masks):
                    img = o[b.offsets[i]:b.offsets[i + 1]].reshape(side, side)
                    want = np.where(mk != 0, full, 0.0)
                    what = "%s fs=%d %s placement %d" % ("fp64" if use_double else "fp32", fs, convolver, i)
                    assert np.all(img[want == 0] == 0), what
                    nz = want != 0
                    assert not nz.any() or np.max(np.abs(img[nz] - want[nz]) / np.abs(want[nz])) <= 1e-4, what
