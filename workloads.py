"""Seeded synthetic workloads of the benchmark configurations.

No public dataset is involved: every input is drawn here with numpy's PCG64,
seed 1000 + configuration number. A workload is a list of model specs in the
form tests/golden/cases.py uses ({"width", "height", "psf", "profiles":
[(kind, params), ...]}), convertible to libprofit_gb300.Model objects or
oracle cases.

  cfg1  one 100x100 model: sersic (xcen 50.3, ycen 50.7, mag 15, re 8, nser 4,
        ang 30, axrat 0.6) convolved with a 15x15 Moffat PSF (fwhm 3, con 2.5).
  cfg2  one 1000x1000 model: sersic bulge (n 4, re 15, axrat 0.8, mag 16,
        ang U[0,180]) + sersic disk (n 1, re 60, axrat 0.35, ang 72, box 0.1,
        mag 15) + sky (bg 1e-3, not convolved); centres U[480,520]; 51x51
        Moffat PSF (fwhm 3.5, con 2.5).
  cfg3  4096 models, side round(exp(U[ln 64, ln 512])), 1-3 profiles drawn
        uniformly from the six radial kinds; nser U[0.5,8], re
        exp(N(ln 6, 0.6)), axrat U[0.1,1], ang U[0,180], box U[-0.3,0.3],
        mag U[14,22], centres U[0, side]; profile-specific parameters are the
        reference constructors' defaults scaled by re (coresersic rb = re,
        a = b = 1; moffat fwhm = 3 re, con 2; ferrer rout = 3 re, a = b = 1;
        king rc = re, rt = 3 re, a = 2; brokenexp h1 = h2 = rb = re, a = 1);
        a Moffat PSF per model, odd side in [15, 41], fwhm U[2,5], con U[1.5,4].
  cfg4  1024 models of 256x256: sersic bulge (nser U[2,6]) + sersic disk
        (nser U[0.7,1.3]), other parameters as cfg3; one 25x25 Moffat PSF
        (fwhm 3, con 2.5).
  cfg5  one 4096x4096 model with 10,000 profiles (60/15/10/5/5/5 % sersic /
        coresersic / moffat / ferrer / king / brokenexp), cfg3 distributions
        with mag U[16,25] and centres U[0,4096], plus a sky; 101x101 Moffat PSF.
Every radial profile is convolved (convolve = 1); the sky is not.
"""
import numpy as np

RADIAL = ["sersic", "coresersic", "moffat", "ferrer", "king", "brokenexp"]


def _rng(cfg):
    return np.random.Generator(np.random.PCG64(1000 + cfg))


def moffat_psf(size, fwhm, con):
    """A centred size x size Moffat PSF rendered from the Moffat profile
    formula at pixel centres, normalised to unit sum (set_psf normalises
    again)."""
    c = size / 2.0
    y, x = np.mgrid[0:size, 0:size] + 0.5
    rscale = fwhm / (2 * np.sqrt(2 ** (1 / con) - 1))
    img = (1 + ((x - c) ** 2 + (y - c) ** 2) / rscale ** 2) ** (-con)
    return img / img.sum()


def _extras(kind, re, rng, nser):
    if kind == "sersic":
        return dict(re=re, nser=nser)
    if kind == "coresersic":
        return dict(re=re, rb=re, nser=nser, a=1.0, b=1.0)
    if kind == "moffat":
        return dict(fwhm=3 * re, con=2.0)
    if kind == "ferrer":
        return dict(rout=3 * re, a=1.0, b=1.0)
    if kind == "king":
        return dict(rc=re, rt=3 * re, a=2.0)
    return dict(h1=re, h2=re, rb=re, a=1.0)


def _radial(kind, rng, side_x, side_y, mag_lo=14.0, mag_hi=22.0, nser=None):
    re = float(np.exp(rng.normal(np.log(6.0), 0.6)))
    n = float(rng.uniform(0.5, 8.0)) if nser is None else nser
    p = dict(xcen=float(rng.uniform(0, side_x)), ycen=float(rng.uniform(0, side_y)),
             mag=float(rng.uniform(mag_lo, mag_hi)), ang=float(rng.uniform(0, 180)),
             axrat=float(rng.uniform(0.1, 1.0)), box=float(rng.uniform(-0.3, 0.3)), convolve=True)
    p.update(_extras(kind, re, rng, n))
    return (kind, p)


def cfg1():
    return [dict(width=100, height=100, psf=moffat_psf(15, 3.0, 2.5), profiles=[
        ("sersic", dict(xcen=50.3, ycen=50.7, mag=15.0, re=8.0, nser=4.0, ang=30.0, axrat=0.6, box=0.0,
                        convolve=True))])]


def cfg2():
    rng = _rng(2)
    bulge = dict(xcen=float(rng.uniform(480, 520)), ycen=float(rng.uniform(480, 520)), mag=16.0, re=15.0,
                 nser=4.0, ang=float(rng.uniform(0, 180)), axrat=0.8, box=0.0, convolve=True)
    disk = dict(xcen=float(rng.uniform(480, 520)), ycen=float(rng.uniform(480, 520)), mag=15.0, re=60.0,
                nser=1.0, ang=72.0, axrat=0.35, box=0.1, convolve=True)
    return [dict(width=1000, height=1000, psf=moffat_psf(51, 3.5, 2.5), convolver="fft",
                 profiles=[("sersic", bulge), ("sersic", disk), ("sky", dict(bg=1e-3))])]


def cfg3(n_models=4096):
    rng = _rng(3)
    models = []
    for _ in range(n_models):
        side = int(round(float(np.exp(rng.uniform(np.log(64), np.log(512))))))
        n_prof = int(rng.integers(1, 4))
        profs = [_radial(RADIAL[int(rng.integers(0, 6))], rng, side, side) for _ in range(n_prof)]
        psf_side = 15 + 2 * int(rng.integers(0, 14))
        psf = moffat_psf(psf_side, float(rng.uniform(2, 5)), float(rng.uniform(1.5, 4)))
        models.append(dict(width=side, height=side, psf=psf, profiles=profs))
    return models


def cfg4(n_models=1024):
    rng = _rng(4)
    psf = moffat_psf(25, 3.0, 2.5)
    models = []
    for _ in range(n_models):
        bulge = _radial("sersic", rng, 256, 256, nser=float(rng.uniform(2, 6)))
        disk = _radial("sersic", rng, 256, 256, nser=float(rng.uniform(0.7, 1.3)))
        models.append(dict(width=256, height=256, psf=psf, profiles=[bulge, disk]))
    return models


def cfg5(n_profiles=10000):
    rng = _rng(5)
    kinds = rng.choice(len(RADIAL), size=n_profiles, p=[0.6, 0.15, 0.10, 0.05, 0.05, 0.05])
    profs = [_radial(RADIAL[int(k)], rng, 4096, 4096, mag_lo=16.0, mag_hi=25.0) for k in kinds]
    profs.append(("sky", dict(bg=1e-3)))
    return [dict(width=4096, height=4096, psf=moffat_psf(101, 3.0, 2.5), convolver="fft", profiles=profs)]


CONFIGS = {1: cfg1, 2: cfg2, 3: cfg3, 4: cfg4, 5: cfg5}


def to_model(spec, env=None):
    """A libprofit_gb300.Model from a spec."""
    import libprofit_gb300 as pg
    m = pg.Model(spec["width"], spec["height"])
    m.set_magzero(spec.get("magzero", 0.0))
    if spec.get("convolver") in ("fft", "brute", "auto"):
        m.set_convolver(spec["convolver"])
    if spec.get("psf") is not None:
        m.set_psf(spec["psf"])
    if spec.get("mask") is not None:
        m.set_mask(spec["mask"])
        m.set_adjust_mask(spec.get("adjust_mask", True))
    if env is not None:
        m.set_cuda_env(env)
    for kind, params in spec["profiles"]:
        p = m.add_profile(kind)
        for k, v in params.items():
            p.parameter(k, bool(v) if k in ("convolve", "rough", "adjust", "rescale_flux") else
                        (int(v) if k in ("resolution", "max_recursions") else float(v)))
    return m


def to_oracle_case(spec):
    from oracle import oracle as O
    return O.Case(spec["width"], spec["height"], spec["profiles"], psf=spec.get("psf"),
                  magzero=spec.get("magzero", 0.0), mask=spec.get("mask"),
                  adjust_mask=spec.get("adjust_mask", True))


def param_matrix(specs):
    """The batch's parameter slots (n_profiles x 12), in model order."""
    import libprofit_gb300 as pg
    rows = []
    for s in specs:
        for kind, params in s["profiles"]:
            p = pg.Profile(kind)
            for k, v in params.items():
                if k not in ("convolve", "rough", "adjust", "rescale_flux", "resolution", "max_recursions"):
                    p.parameter(k, float(v))
            rows.append([p.desc.par[i] for i in range(12)])
    return np.array(rows, dtype=np.float64)


def gradient_scales(specs, par, images, data, sigma, env64, h_rel=1e-6, n_par=8):
    """Two scales of each chi^2 gradient component, from central differences
    (h = h_rel x |par|, at least h_rel x 1e-3) of the plain FP64 path at the
    parameters `par` (n_profiles x 12, batch order of `specs`):
      sum_p |c_p dm_p/dpar|, c = 2 (m - d) / sigma^2: the sum the gradient is;
      sum_p 2 |m_p dm_p/dpar| / sigma_p^2: its sensitivity to relative errors
      of the model image m itself.
    An FP32 gradient carries rounding of a few units of 2^-24 on the first
    (its own arithmetic) and on the second times the FP32 image's relative
    error, whatever the component's own size. `images`, `data`, `sigma`: the
    models' FP64 output images back to back (numpy, float64).

    Returns (scale_c, scale_m, same_tree), each n_profiles x n_par: same_tree
    is False where the +-h images of a parameter do not keep the subsampling
    tree (per-level counts differ from the unperturbed model's), so that the
    difference is not a derivative there."""
    import torch
    import libprofit_gb300 as pg
    first = np.cumsum([0] + [len(s["profiles"]) for s in specs])
    scale_c = np.zeros((int(first[-1]), n_par))
    scale_m = np.zeros((int(first[-1]), n_par))
    same = np.ones((int(first[-1]), n_par), dtype=bool)
    out_off = np.cumsum([0] + [s["width"] * s["height"] for s in specs])
    for i, s in enumerate(specs):
        n = len(s["profiles"])
        p0 = par[first[i]:first[i + 1]]
        rows, hs = [p0], []
        for j in range(n):
            for k in range(n_par):
                h = h_rel * max(abs(p0[j, k]), 1e-3)
                hs.append(h)
                for sgn in (1.0, -1.0):
                    q = p0.copy()
                    q[j, k] += sgn * h
                    rows.append(q)
        b = pg.Batch([to_model(s, env64) for _ in rows], env64)
        b.set_params(np.concatenate(rows))
        b.record_depth(True)
        img = torch.zeros(b.total_pixels, dtype=torch.float64, device="cuda")
        b.forward(img)
        b.check()
        im = img.cpu().numpy().reshape(len(rows), -1)
        counts = [c for _, c in b.depth()]
        b.close()
        a, z = out_off[i], out_off[i + 1]
        cot = 2 * (images[a:z] - data[a:z]) / sigma[a:z] ** 2
        msens = 2 * np.abs(images[a:z]) / sigma[a:z] ** 2
        q = 0
        for j in range(n):
            for k in range(n_par):
                up, dn = 1 + 2 * q, 2 + 2 * q
                dm = np.abs(im[up] - im[dn]) / (2 * hs[q])
                scale_c[first[i] + j, k] = np.sum(np.abs(cot) * dm)
                scale_m[first[i] + j, k] = np.sum(msens * dm)
                same[first[i] + j, k] = all(np.array_equal(counts[r * n + jj], counts[jj])
                                            for r in (up, dn) for jj in range(n))
                q += 1
    return scale_c, scale_m, same
