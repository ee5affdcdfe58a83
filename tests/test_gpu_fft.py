"""FFT convolution (GPU).

The reference's FFTConvolver (src/convolve.cpp:233-312) gives, for the pixels
Model::evaluate keeps, the same linear convolution as its brute-force
convolvers up to the FFT's rounding, which is absolute and proportional to
the image's peak. Bars:
  * FP64 FFT against the reference's golden images (brute-force convolved):
    |err| <= 1e-12 x peak everywhere, and <= 1e-10 relative for pixels above
    1e-3 x peak;
  * FP32 FFT against the FP32 direct convolution of the same models:
    |err| <= 2e-6 x peak everywhere, <= 1e-4 relative above 1e-3 x peak;
  * the 1000 x 1000 model with a 51 x 51 PSF (the automatic choice takes the
    FFT) against the FP64 path: flux <= 1e-5 relative, pixels above 1e-3 x peak
    <= 1e-4 relative.
"""
import numpy as np
import pytest

from tests.golden.load import load
from tests.helpers import product_model

pytestmark = pytest.mark.gpu

GOLDEN = load()
CONVOLVED = [n for n in sorted(GOLDEN) if any(p[1].get("convolve") for p in GOLDEN[n]["spec"]["profiles"])]


@pytest.fixture(scope="module")
def envs():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    return pg.get_cuda_environment(0, use_double=True), pg.get_cuda_environment(0, use_double=False)


def _check(img, ref, abs_tol, rel_tol, floor=1e-3):
    peak = np.abs(ref).max()
    if peak == 0:  # everything masked out
        assert np.all(img == 0)
        return
    assert np.max(np.abs(img - ref)) <= abs_tol * peak
    bright = np.abs(ref) > floor * peak
    rel = np.abs(img[bright] - ref[bright]) / np.abs(ref[bright])
    assert rel.max() <= rel_tol, rel.max()


@pytest.mark.parametrize("name", CONVOLVED)
def test_fft_fp64_matches_reference(envs, name):
    env64, _ = envs
    entry = GOLDEN[name]
    m = product_model(entry["spec"], entry["psf"], env64)
    m.set_convolver("fft")
    _check(m.evaluate(), entry["image"], 1e-12, 1e-10)


@pytest.mark.parametrize("name", CONVOLVED)
def test_fft_fp32_matches_direct(envs, name):
    _, env32 = envs
    entry = GOLDEN[name]
    a = product_model(entry["spec"], entry["psf"], env32)
    a.set_convolver("fft")
    b = product_model(entry["spec"], entry["psf"], env32)
    b.set_convolver("brute")
    _check(a.evaluate(), b.evaluate(), 2e-6, 1e-4)


FFT32_LENGTHS = [64, 96, 128, 160, 192, 256, 288, 320, 384, 512, 576, 640, 768, 1024, 1152, 1280, 1536, 2048,
                 2304, 2560, 3072, 4096, 4608, 5120, 6144, 8192]


@pytest.mark.parametrize("n", FFT32_LENGTHS)
def test_fft32_every_length(envs, n):
    """Every single-precision transform length (2^a, 3, 5, 9 x 2^a): a model
    of width (or height) n - 15 with a 15 x 15 PSF needs exactly n points
    (crop + psf) and gets that length; its FFT convolution against the direct
    one, at the FP32 FFT bars. Lengths up to 2304 square, longer ones on thin
    models along either axis."""
    import workloads as W
    _, env32 = envs
    k = 15
    shapes = [(n - k, n - k)] if n <= 2304 else [(n - k, 40), (40, n - k)]
    for w, h in shapes:
        spec = dict(width=w, height=h, psf=W.moffat_psf(k, 3.0, 2.5), profiles=[
            ("sersic", dict(xcen=0.4 * w, ycen=0.55 * h, mag=15.0, re=max(3.0, min(w, h) / 8), nser=2.5, ang=30.0,
                            axrat=0.7, box=0.0, convolve=True))])
        a = W.to_model(dict(spec, convolver="fft"), env32)
        b = W.to_model(dict(spec, convolver="brute"), env32)
        _check(a.evaluate(), b.evaluate(), 2e-6, 1e-4)


def test_fft_batch_mixed_methods(envs):
    """Models with FFT and direct convolution in one batch render as alone."""
    import torch
    import libprofit_gb300 as pg
    import workloads as W
    _, env32 = envs
    specs = W.cfg3(24)
    models = []
    for i, s in enumerate(specs):
        m = W.to_model(s, env32)
        m.set_convolver("fft" if i % 2 else "brute")
        models.append(m)
    b = pg.Batch(models, env32)
    out = torch.zeros(b.total_pixels, dtype=torch.float32, device="cuda")
    b.forward(out)
    b.check()
    o = out.cpu().numpy()
    for i, m in enumerate(models):
        w, h = b.dims[i]
        img = o[b.offsets[i]:b.offsets[i + 1]].reshape(h, w).astype(np.float64)
        assert np.array_equal(img, m.evaluate())


def test_large_psf_auto_fft(envs):
    """1000 x 1000, bulge + disk + sky, 51 x 51 Moffat PSF."""
    import workloads as W
    env64, env32 = envs
    spec = W.cfg2()[0]
    spec = dict(spec, convolver="auto")
    ref = W.to_model(spec, env64).evaluate()
    img = W.to_model(spec, env32).evaluate()
    assert abs(img.sum() - ref.sum()) <= 1e-5 * abs(ref.sum())
    _check(img, ref, 2e-6, 1e-4)


@pytest.mark.parametrize("use_double,width", [(True, 4100), (False, 8190)])
def test_fft_longer_than_transforms_takes_direct(envs, use_double, width):
    """A model whose FFT would exceed the longest transform (4096 points per
    side in double precision, 8192 in single) is convolved directly: the
    same cropped image as requesting the direct convolution, bit for bit."""
    import workloads as W
    env = envs[0] if use_double else envs[1]
    spec = dict(width=width, height=40, psf=W.moffat_psf(15, 3.0, 2.5), profiles=[
        ("sersic", dict(xcen=0.3 * width, ycen=20.0, mag=15.0, re=12.0, nser=2.0, ang=20.0, axrat=0.6, box=0.0,
                        convolve=True))])
    a = W.to_model(dict(spec, convolver="fft"), env).evaluate()
    b = W.to_model(dict(spec, convolver="brute"), env).evaluate()
    assert np.array_equal(a, b)
    assert a.max() > 0
