"""Adjoint of the coresersic, moffat, ferrer, king and brokenexp profiles
against central finite differences of the FP64 oracle (GPU).

One 64 x 64 model per profile kind (the profile convolved by a 15 x 15 Moffat
PSF, plus a sky), round and boxy; data = the oracle's image at parameters
perturbed by 5 % plus noise; chi^2 = sum ((model - data) / sigma)^2. Every
parameter of the profile (xcen, ycen, mag, ang, axrat, box and the kind's own)
and the sky's bg must match central differences of the oracle's chi^2 with
h = 1e-6 relative, by the criterion of tests/helpers.py (that of the sersic
adjoint test):
  |g - fd| <= 1e-4 |fd| + 1e-14 sum|c m| / h
              (+ 2e-6 sum|c dm/dpar| + 2e-6 sum 2|m dm/dpar| / sigma^2 in FP32)
Parameters whose finite difference is not that of a smooth function are
excluded (at most two per case): those whose +-h changes the oracle's
subsampling tree (level counts), which the adjoint holds fixed, and those
whose difference quotient moves by more than 2e-5 relative when h shrinks ten
times -- a sub-point near the cusp of a coresersic (f ~ r^-b at its centre)
makes the h = 1e-6 quotient depart from the derivative by up to a few 1e-4,
while the quotients of smaller steps converge to the adjoint's value.
A batch holding all the models (and a sersic one, so that the twelve-slot
kernels also run the sersic's terms) gives every model's gradient as the
single-model batches do.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIDE = 64
MAGZERO = 25.0
GEOM = ("xcen", "ycen", "mag", "ang", "axrat", "box")
OWN = {
    "coresersic": dict(re=8.0, nser=2.5, rb=2.0, a=3.0, b=0.5),
    "moffat": dict(fwhm=6.0, con=2.5),
    "ferrer": dict(rout=20.0, a=1.5, b=0.6),
    "king": dict(rc=4.0, rt=25.0, a=2.0),
    "brokenexp": dict(h1=5.0, h2=3.0, rb=10.0, a=1.0),
}
ORDER = {k: list(GEOM) + list(v) for k, v in OWN.items()}
# (kind, box, overrides of OWN): round and boxy, plus a coresersic without the
# central cusp (b = 0), whose centre derivatives the finite differences can check
CASES = [(kind, box, None) for kind in OWN for box in (0.0, 0.2)] + [("coresersic", 0.1, dict(b=0.0))]
IDS = ["%s-box%g%s" % (k, b, "-flat" if o else "") for k, b, o in CASES]


def _truth(kind, box, over):
    p = dict(xcen=31.3, ycen=29.6, mag=15.0, ang=33.0, axrat=0.7, box=box, convolve=True)
    p.update(OWN[kind])
    p.update(over or {})
    return [(kind, p), ("sky", dict(bg=1.0))]


def _with(profiles, i, k, v):
    from tests.helpers import with_param
    return with_param(profiles, i, k, v)


def _problem(O, kind, box, over):
    import workloads as W
    rng = np.random.default_rng(sum(map(ord, kind)) * 10 + int(round(box * 10)))
    psf = W.moffat_psf(15, 3.0, 2.5)
    truth = _truth(kind, box, over)
    data, _, _ = O.evaluate(O.Case(SIDE, SIDE, truth, psf=psf, magzero=MAGZERO))
    perturbed = []
    for k_, p in truth:
        q = dict(p)
        for k in q:
            if k in ("convolve", "box") or q[k] == 0:
                continue
            q[k] = q[k] + 0.3 * rng.normal() if k in ("xcen", "ycen") else q[k] * (1 + 0.05 * rng.normal())
        if k_ != "sky":
            q["axrat"] = min(q["axrat"], 1.0)
            q["box"] = box + (0.02 * rng.normal() if box else 0.0)
        perturbed.append((k_, q))
    sigma = 0.01 * data.max()
    data = data + rng.normal(0, sigma, data.shape)
    return psf, perturbed, data, np.full_like(data, sigma)


def _chi2(O, psf, profiles, data, sigma):
    img, _, counts = O.evaluate(O.Case(SIDE, SIDE, profiles, psf=psf, magzero=MAGZERO))
    return float(np.sum(((img - data) / sigma) ** 2)), counts


def _render(O, psf):
    def render(p):
        img, _, counts = O.evaluate(O.Case(SIDE, SIDE, p, psf=psf, magzero=MAGZERO))
        return img, counts
    return render


def _fd(O, psf, profiles, data, sigma):
    from tests.helpers import fd_gradients
    names = [(0, k) for k in ORDER[profiles[0][0]]] + [(1, "bg")]
    return fd_gradients(_render(O, psf), profiles, names, data, sigma, smooth=True)[1]


def _slot(kind, k):
    if k == "bg":
        return 6
    order = ORDER[kind]
    return order.index(k)  # par[0..5] geometric, par[6..] the kind's own, in registration order


@pytest.fixture(scope="module")
def problems(oracle_lib):
    out = {}
    for kind, box, over in CASES:
        psf, profiles, data, sigma = _problem(oracle_lib, kind, box, over)
        out[(kind, box, bool(over))] = (psf, profiles, data, sigma, _fd(oracle_lib, psf, profiles, data, sigma))
    return out


def _models(pg, W, env, specs):
    return [W.to_model(dict(width=SIDE, height=SIDE, psf=psf, profiles=profiles, magzero=MAGZERO), env)
            for psf, profiles in specs]


def _gpu_grads(specs, datas, sigmas, use_double):
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    env = pg.get_cuda_environment(0, use_double=use_double)
    models = _models(pg, W, env, specs)
    b = pg.Batch(models, env)
    b.enable_adjoint()
    dt = torch.float64 if use_double else torch.float32
    img = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
    d = torch.tensor(np.concatenate([x.ravel() for x in datas]), dtype=dt, device="cuda")
    s = torch.tensor(np.concatenate([x.ravel() for x in sigmas]), dtype=dt, device="cuda")
    chi2 = torch.zeros(len(models), dtype=torch.float64, device="cuda")
    n_prof = sum(len(p) for _, p in specs)
    grad = torch.zeros(n_prof * 12, dtype=torch.float64, device="cuda")
    b.forward_backward(img, d, s, chi2, grad)
    b.check()
    return chi2.cpu().numpy(), grad.cpu().numpy().reshape(n_prof, 12)


@pytest.mark.parametrize("use_double", [True, False])
@pytest.mark.parametrize("kind,box,over", CASES, ids=IDS)
def test_profile_gradient_matches_finite_differences(problems, oracle_lib, kind, box, over, use_double):
    psf, profiles, data, sigma, fd = problems[(kind, box, bool(over))]
    chi2, grad = _gpu_grads([(psf, profiles)], [data], [sigma], use_double)
    chi2_ref, _ = _chi2(oracle_lib, psf, profiles, data, sigma)
    assert abs(chi2[0] - chi2_ref) <= (1e-10 if use_double else 1e-5) * chi2_ref
    checked = skipped = 0
    for (i, k), r in fd.items():
        if not r.usable:
            skipped += 1
            continue
        r.check(grad[i, _slot(kind, k) if i == 0 else 6], not use_double, "%s box %g %s" % (kind, box, k))
        checked += 1
    assert skipped <= 2 and checked >= len(fd) - 2


@pytest.mark.parametrize("use_double", [True, False])
def test_mixed_batch_equals_single_models(problems, use_double):
    import tests.test_gpu_adjoint as S
    from oracle import oracle as O
    specs, datas, sigmas = [], [], []
    for kind, box, over in CASES:
        psf, profiles, data, sigma, _ = problems[(kind, box, bool(over))]
        specs.append((psf, profiles))
        datas.append(data)
        sigmas.append(sigma)
    spsf, sprof, sdata, ssig = S.make_problem(O)
    specs.append((spsf, sprof))
    datas.append(sdata)
    sigmas.append(ssig)
    chi2_all, g_all = _gpu_grads(specs, datas, sigmas, use_double)
    row = 0
    tol = 1e-9 if use_double else 1e-5
    for j, (spec, data, sigma) in enumerate(zip(specs, datas, sigmas)):
        chi2_one, g_one = _gpu_grads([spec], [data], [sigma], use_double)
        n = len(spec[1])
        assert abs(chi2_all[j] - chi2_one[0]) <= tol * chi2_one[0]
        scale = np.abs(g_one).max()
        np.testing.assert_allclose(g_all[row:row + n], g_one, rtol=tol * 100, atol=tol * scale)
        row += n


# The psf profile (a point source, src/psf.cpp:58-145): its stamp's overlaps
# with the image pixels are piecewise linear in the centre, so its xcen and
# ycen gradients are those of the overlap lengths; mag scales it. A sersic
# (convolved) plus two point sources, one convolved and one not, plus a sky.
def _psf_problem(O):
    import workloads as W
    rng = np.random.default_rng(31)
    psf = W.moffat_psf(15, 3.0, 2.5)
    truth = [("sersic", dict(xcen=30.2, ycen=33.7, mag=16.0, re=5.0, nser=2.0, ang=20.0, axrat=0.6, convolve=True)),
             ("psf", dict(xcen=20.37, ycen=22.81, mag=17.0)),
             ("psf", dict(xcen=44.62, ycen=17.29, mag=16.5, convolve=True)),
             ("sky", dict(bg=0.5))]
    data, _, _ = O.evaluate(O.Case(SIDE, SIDE, truth, psf=psf, magzero=MAGZERO))
    perturbed = [(k, dict(p)) for k, p in truth]
    perturbed[1][1].update(xcen=20.61, ycen=22.55, mag=17.2)
    perturbed[2][1].update(xcen=44.43, ycen=17.48, mag=16.3)
    sigma = 0.01 * data.max()
    data = data + rng.normal(0, sigma, data.shape)
    return psf, perturbed, data, np.full_like(data, sigma)


@pytest.mark.parametrize("use_double", [True, False])
def test_psf_profile_gradient_matches_finite_differences(oracle_lib, use_double):
    O = oracle_lib
    psf, profiles, data, sigma = _psf_problem(O)
    chi2, grad = _gpu_grads([(psf, profiles)], [data], [sigma], use_double)
    chi2_ref, _ = _chi2(O, psf, profiles, data, sigma)
    assert abs(chi2[0] - chi2_ref) <= (1e-10 if use_double else 1e-5) * chi2_ref
    from tests.helpers import fd_gradients
    slots = {"xcen": 0, "ycen": 1, "mag": 2}
    names = [(i, k) for i in (1, 2) for k in ("xcen", "ycen", "mag")]
    _, fd = fd_gradients(_render(O, psf), profiles, names, data, sigma)
    for (i, k), r in fd.items():
        r.check(grad[i, slots[k]], not use_double, "psf %d %s" % (i, k))


# A Sersic with rescale_flux (src/sersic.cpp:302-325): the flux scale divides
# by P(2n, bn (rscale_max / re)^(1/n)), with rscale_max given (so it moves
# with re and nser through x) and derived by adjust (a ceiling: constant
# between its steps).
@pytest.mark.parametrize("use_double", [True, False])
@pytest.mark.parametrize("rscale_max", [6.0, 0.0])
def test_rescale_flux_gradient_matches_finite_differences(oracle_lib, use_double, rscale_max):
    import workloads as W
    O = oracle_lib
    rng = np.random.default_rng(57)
    psf = W.moffat_psf(15, 3.0, 2.5)
    sersic = dict(xcen=31.1, ycen=30.4, mag=16.0, re=6.0, nser=2.6, ang=35.0, axrat=0.65, box=0.05, convolve=True,
                  rescale_flux=True, rscale_max=rscale_max)
    truth = [("sersic", sersic), ("sky", dict(bg=0.3))]
    data, _, _ = O.evaluate(O.Case(SIDE, SIDE, truth, psf=psf, magzero=MAGZERO))
    profiles = _with(_with(_with(truth, 0, "re", 6.4), 0, "nser", 2.4), 0, "xcen", 31.5)
    sigma = np.full_like(data, 0.01 * data.max())
    data = data + rng.normal(0, sigma[0, 0], data.shape)
    chi2, grad = _gpu_grads([(psf, profiles)], [data], [sigma], use_double)
    chi2_ref, _ = _chi2(O, psf, profiles, data, sigma)
    assert abs(chi2[0] - chi2_ref) <= (1e-10 if use_double else 1e-5) * chi2_ref
    from tests.helpers import fd_gradients
    slots = {"xcen": 0, "mag": 2, "axrat": 4, "re": 6, "nser": 7}
    _, fd = fd_gradients(_render(O, psf), profiles, [(0, k) for k in slots], data, sigma)
    checked = 0
    for (_, k), r in fd.items():
        if not r.usable:
            continue
        r.check(grad[0, slots[k]], not use_double, k)
        checked += 1
    assert checked >= 4
