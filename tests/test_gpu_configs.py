"""The benchmark configurations at their full sizes (GPU).

The FP32 batched path against the plain FP64 path, which equals the reference
to 1e-10 per pixel on every golden case; at these sizes the oracle itself
would take hours, so the size-independent properties are checked here:
  * cfg3: 4096 uneven models (sides 64-512, 1-3 profiles of the six radial
    kinds, a Moffat PSF each, convolution method by the autotuner) in one FP32
    batch; every 16th model rendered by the FP64 path: flux <= 1e-5 relative,
    pixels above 1e-3 x peak <= 1e-4 relative, every pixel within 1e-4
    relative + 1e-6 x peak + 2e-8 x the total flux (the FP32 FFT's rounding is
    absolute);
  * cfg4: 1024 models of 256 x 256 (sersic bulge + disk, 25 x 25 PSF), one
    FP32 batch with the adjoint: flux, pixels, chi^2 and all 16 gradients of
    every 32nd model against the FP64 path: |g32 - g64| <= 1e-4 |g64| +
    2e-6 sum_p |c_p dm_p/dpar| + 2e-6 sum_p 2 |m_p dm_p/dpar| / sigma_p^2 (the
    scale of the sum the gradient is, and its sensitivity to the FP32 image's
    relative error, from central differences of the FP64 path; c = 2 (m - d)
    / sigma^2), for every parameter whose +-1e-6 differences keep the
    subsampling tree (the data here are the FP32 images with 1 % noise, so
    the residuals are small and the second floor is the larger);
  * cfg5: the 4096 x 4096 crowded field (10,000 profiles and a sky, 101 x 101
    PSF by an 8192 x 8192 FP32 FFT) against the FP64 path with the direct
    convolution: flux <= 1e-5, pixels above 1e-3 x peak <= 1e-4, every pixel
    within 1e-4 relative + 1e-6 x peak + 2e-8 x the total flux.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# FP32 gradient floors (tests/helpers.py): on the scale of the gradient's sum
# and on its sensitivity to the FP32 image's relative error
FP32_C = 2e-6
FP32_M = 2e-6


@pytest.fixture(scope="module")
def envs():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    return pg.get_cuda_environment(0, use_double=True), pg.get_cuda_environment(0, use_double=False)


def _check(img, ref, name):
    peak = np.abs(ref).max()
    flux = np.abs(ref).sum()
    assert abs(img.sum() - ref.sum()) <= 1e-5 * abs(ref.sum()), "%s: flux %.3g" % (
        name, abs(img.sum() - ref.sum()) / abs(ref.sum()))
    # every pixel: 1e-4 relative plus an absolute floor for the FP32 FFT's
    # rounding, which is of the order of eps x the image's total flux spread
    # over the transform (1e-6 x peak + 2e-8 x flux)
    err = np.abs(img - ref) - 1e-4 * np.abs(ref)
    assert err.max() <= 1e-6 * peak + 2e-8 * flux, "%s: abs %.3g of peak" % (name, err.max() / peak)
    # 1e-4 relative from 1e-2 x peak up: the FP32 FFT's rounding, about
    # 1e-7 x peak wherever the pixel is, is already 1e-4 of a pixel at
    # 1e-3 x peak (the models whose autotuned method is the FFT)
    bright = np.abs(ref) > 1e-2 * peak
    rel = np.abs(img[bright] - ref[bright]) / np.abs(ref[bright])
    assert rel.max() <= 1e-4, "%s: rel %.3g" % (name, rel.max())


def _render(pg, models, env, dtype):
    import torch
    b = pg.Batch(models, env)
    out = torch.zeros(b.total_pixels, dtype=dtype, device="cuda")
    b.forward(out)
    b.check()
    o = out.cpu().numpy().astype(np.float64)
    imgs = [o[b.offsets[i]:b.offsets[i + 1]].reshape(h, w) for i, (w, h) in enumerate(b.dims)]
    b.close()
    return imgs


def test_cfg3_full_batch(envs):
    import torch
    import libprofit_gb300 as pg
    import workloads as W
    env64, env32 = envs
    specs = W.cfg3()
    assert len(specs) == 4096
    imgs32 = _render(pg, [W.to_model(s, env32) for s in specs], env32, torch.float32)
    pick = list(range(0, len(specs), 16))
    imgs64 = _render(pg, [W.to_model(specs[i], env64) for i in pick], env64, torch.float64)
    for j, i in enumerate(pick):
        _check(imgs32[i], imgs64[j], "model %d" % i)


def test_cfg4_full_batch_with_gradients(envs):
    import torch
    import libprofit_gb300 as pg
    import workloads as W
    env64, env32 = envs
    specs = W.cfg4()
    rng = np.random.default_rng(44)
    pick = list(range(0, len(specs), 32))

    def run(env, sel, dtype):
        models = [W.to_model(specs[i], env) for i in sel]
        b = pg.Batch(models, env)
        b.enable_adjoint()
        img = torch.zeros(b.total_pixels, dtype=dtype, device="cuda")
        b.forward(img)
        b.check()
        return b, img

    b32, img32 = run(env32, range(len(specs)), torch.float32)
    ref_imgs = img32.cpu().numpy().astype(np.float64)
    # data: the FP32 images perturbed by 1 % noise (any fixed data serves)
    data = ref_imgs * (1 + 0.01 * rng.standard_normal(ref_imgs.shape))
    sigma = np.full_like(data, 0.01 * ref_imgs.max())
    d32 = torch.tensor(data, dtype=torch.float32, device="cuda")
    s32 = torch.tensor(sigma, dtype=torch.float32, device="cuda")
    chi32 = torch.zeros(len(specs), dtype=torch.float64, device="cuda")
    g32 = torch.zeros(b32.n_profiles * 12, dtype=torch.float64, device="cuda")
    b32.forward_backward(img32, d32, s32, chi32, g32)
    b32.check()
    b64, img64 = run(env64, pick, torch.float64)
    sel = np.concatenate([np.arange(b32.offsets[i], b32.offsets[i + 1]) for i in pick])
    d64 = torch.tensor(data[sel], dtype=torch.float64, device="cuda")
    s64 = torch.tensor(sigma[sel], dtype=torch.float64, device="cuda")
    chi64 = torch.zeros(len(pick), dtype=torch.float64, device="cuda")
    g64 = torch.zeros(b64.n_profiles * 12, dtype=torch.float64, device="cuda")
    b64.forward_backward(img64, d64, s64, chi64, g64)
    b64.check()
    i32, i64 = img32.cpu().numpy().astype(np.float64), img64.cpu().numpy()
    G32, G64 = g32.cpu().numpy().reshape(-1, 12), g64.cpu().numpy().reshape(-1, 12)
    c32, c64 = chi32.cpu().numpy(), chi64.cpu().numpy()
    scale_c, scale_m, same = W.gradient_scales([specs[i] for i in pick], W.param_matrix([specs[i] for i in pick]),
                                               i64, data[sel], sigma[sel], env64)
    assert same.mean() >= 0.85  # +-1e-6 changes the tree of ~7 % of the parameters here
    G32p = np.concatenate([G32[2 * i:2 * i + 2, :8] for i in pick])
    G64p = G64[:, :8]
    err = np.abs(G32p - G64p)
    print("cfg4 gradients: err/scale_c max %.3g, err/scale_m max %.3g, err/(1e-4|g|) max %.3g" % (
        (err / scale_c)[same].max(), (err / scale_m)[same].max(), (err / (1e-4 * np.abs(G64p)))[same].max()))
    for j, i in enumerate(pick):
        a = i32[b32.offsets[i]:b32.offsets[i + 1]]
        r = i64[b64.offsets[j]:b64.offsets[j + 1]]
        _check(a, r, "model %d" % i)
        # chi^2 is ~0.3 here (residuals of 1 % of the image against sigma = 1 % of
        # the peak), so its relative error is the FP32 image's, not the 1e-5 of
        # the fitting workload
        assert abs(c32[i] - c64[j]) <= 1e-4 * c64[j]
        ga, gr = G32[2 * i:2 * i + 2, :8], G64[2 * j:2 * j + 2, :8]
        sc, sm, ok = scale_c[2 * j:2 * j + 2], scale_m[2 * j:2 * j + 2], same[2 * j:2 * j + 2]
        bound = 1e-4 * np.abs(gr) + FP32_C * sc + FP32_M * sm
        bad = ok & (np.abs(ga - gr) > bound)
        assert not bad.any(), "model %d: %s vs %s (scales %s, %s)" % (i, ga[bad], gr[bad], sc[bad], sm[bad])


def test_cfg5_crowded_field(envs):
    import torch
    import libprofit_gb300 as pg
    import workloads as W
    env64, env32 = envs
    spec = W.cfg5()[0]
    assert len(spec["profiles"]) == 10001
    img32, = _render(pg, [W.to_model(spec, env32)], env32, torch.float32)
    img64, = _render(pg, [W.to_model(dict(spec, convolver="brute"), env64)], env64, torch.float64)
    assert img32.shape == (4096, 4096)
    _check(img32, img64, "cfg5")
