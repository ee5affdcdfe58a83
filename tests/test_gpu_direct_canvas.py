"""The unconvolved ("direct") image of models whose profiles all convolve (GPU).

Model::produce_image draws unconvolved profiles into the model image and
adds the convolution of the others to it (src/model.cpp:322-360). Here a
model all of whose profiles convolve has an all-zero direct image: the
single-precision evaluation leaves it unwritten and the convolution and FFT
passes take zeros instead of reading it. A batch mixes such models with
models that draw an unconvolved Sersic profile or a sky, on the direct and
the FFT convolution, and each model's image must equal its rendering alone
bit for bit, and the plain FP64 path's within the FP32 bars (flux <= 1e-5
relative; pixels above 1e-3 x peak <= 1e-4 relative for the direct
convolution, absolute <= 2e-6 x peak for the FFT).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def envs():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    return pg.get_cuda_environment(0, use_double=True), pg.get_cuda_environment(0, use_double=False)


def _specs():
    import workloads as W
    psf = W.moffat_psf(15, 3.0, 2.5)
    specs = []
    for i in range(8):
        w, h = 96 + 8 * i, 80 + 4 * i
        bulge = dict(xcen=w * 0.45, ycen=h * 0.55, mag=15.0, re=6.0 + i, nser=3.0, ang=30.0 + 10 * i, axrat=0.7,
                     convolve=True)
        disk = dict(xcen=w * 0.52, ycen=h * 0.48, mag=15.5, re=12.0, nser=1.0, ang=100.0, axrat=0.4,
                    convolve=i % 4 != 1)  # models 1 and 5 draw the disk unconvolved
        profiles = [("sersic", bulge), ("sersic", disk)]
        if i % 4 == 2:  # models 2 and 6 add a sky, drawn unconvolved
            profiles.append(("sky", dict(bg=0.05)))
        specs.append(dict(width=w, height=h, psf=psf, profiles=profiles,
                          convolver="fft" if i % 2 else "brute"))
    return specs


def test_batch_with_and_without_direct_images(envs):
    import torch
    import libprofit_gb300 as pg
    import workloads as W
    env64, env32 = envs
    specs = _specs()
    models = [W.to_model(s, env32) for s in specs]
    b = pg.Batch(models, env32)
    out = torch.zeros(b.total_pixels, dtype=torch.float32, device="cuda")
    b.forward(out)
    b.check()
    o = out.cpu().numpy()
    for i, (m, s) in enumerate(zip(models, specs)):
        w, h = b.dims[i]
        img = o[b.offsets[i]:b.offsets[i + 1]].reshape(h, w).astype(np.float64)
        assert np.array_equal(img, m.evaluate()), i
        ref = W.to_model(dict(s, convolver="brute"), env64).evaluate()
        assert abs(img.sum() - ref.sum()) <= 1e-5 * abs(ref.sum()), i
        peak = np.abs(ref).max()
        if s["convolver"] == "fft":
            assert np.max(np.abs(img - ref)) <= 2e-6 * peak, i
        else:
            bright = np.abs(ref) > 1e-3 * peak
            assert np.max(np.abs(img[bright] - ref[bright]) / np.abs(ref[bright])) <= 1e-4, i
