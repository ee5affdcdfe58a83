"""Direct convolution over PSF and image shapes (GPU).

The batched direct convolution (conv_kernel) applies a PSF's whole groups of
four columns and then its kw mod 4 remaining columns in a pass of their own,
and unrolls its row loop differently for PSFs shorter and taller than a
block's R output rows; each image size selects a block shape (the one with
the least tile area). Both directions are checked here for PSF widths with
every kw mod 4, heights on both sides of R = 8, odd and even sizes and
asymmetric PSFs, against references that do not use that kernel:
  * forward: the FP32 image against the plain FP64 path (the reference's
    brute-force summation order, pinned to libprofit): flux <= 1e-5
    relative, pixels above 1e-3 x peak <= 1e-4 relative;
  * adjoint: the gradient with respect to each profile's magnitude is, for
    any cotangent c, -0.4 ln(10) <c, that profile's convolved image>
    (flux scales as 10^(-0.4 mag), the subsampling tree does not move), the
    right side taken from the FP64 path's forward image of that profile
    alone: FP64 adjoint <= 1e-10 relative, FP32 adjoint <= 1e-4;
  * the FP32 gradients of every parameter against the FP64 ones:
    <= 1e-3 relative plus 1e-4 of the largest component.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

LN10 = np.log(10.0)
# (PSF width, PSF height, image width, image height): widths cover kw mod 4 =
# 0..3, heights both sides of R = 8; the image sizes are the five block
# shapes' tiles (64 x 128, 56 x 70, 64 x 96, 140 x 56) and ragged sizes
CASES = [
    (1, 1, 64, 128), (2, 3, 56, 70), (3, 2, 64, 96), (4, 4, 140, 56), (5, 7, 61, 47),
    (6, 6, 64, 128), (7, 5, 56, 70), (8, 9, 64, 96), (9, 12, 140, 56), (11, 4, 37, 90),
    (13, 13, 64, 128), (16, 5, 56, 70), (17, 21, 64, 96), (25, 25, 140, 56), (26, 10, 100, 33),
]


def _psf(kw, kh):
    """A normalised, asymmetric (tilted, skewed) PSF: a flipped or transposed
    kernel gives a different image."""
    y, x = np.mgrid[0:kh, 0:kw] + 0.5
    cx, cy = kw * 0.45, kh * 0.55
    sx, sy = max(kw / 4.0, 0.4), max(kh / 3.0, 0.4)
    u, v = (x - cx) / sx, (y - cy) / sy
    p = np.exp(-0.5 * (u * u + v * v + 0.6 * u * v)) * (1.0 + 0.3 * (x / kw) - 0.2 * (y / kh))
    return p / p.sum()


def _profiles(w, h):
    r = min(w, h)
    return [
        ("sersic", dict(xcen=w * 0.47, ycen=h * 0.53, mag=15.0, re=r / 7.0, nser=2.4, ang=38.0, axrat=0.6,
                        box=0.1, convolve=True)),
        ("sersic", dict(xcen=w * 0.52, ycen=h * 0.49, mag=15.5, re=r / 4.0, nser=1.0, ang=115.0, axrat=0.45,
                        convolve=True)),
        ("sky", dict(bg=0.3)),
    ]


@pytest.fixture(scope="module")
def envs():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    return pg.get_cuda_environment(0, use_double=True), pg.get_cuda_environment(0, use_double=False)


def _run(env, use_double, w, h, psf, profiles, cot):
    """Forward image and, for the cotangent, the gradient (profiles x 12)."""
    import torch
    import libprofit_gb300 as pg
    import workloads as W
    m = W.to_model(dict(width=w, height=h, psf=psf, profiles=profiles), env)
    m.set_convolver("brute")
    b = pg.Batch([m], env)
    b.enable_adjoint()
    dt = torch.float64 if use_double else torch.float32
    img = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
    b.forward(img)
    grad = torch.zeros(len(profiles) * 12, dtype=torch.float64, device="cuda")
    c = torch.tensor(cot.ravel(), dtype=dt, device="cuda")
    b.backward(img, cotangent=c, grad=grad)
    b.check()
    info = b.conv_info()
    return (img.cpu().numpy().astype(np.float64).reshape(h, w), grad.cpu().numpy().reshape(len(profiles), 12),
            info)


_SHAPES = set()


@pytest.mark.parametrize("kw,kh,w,h", CASES, ids=["psf%dx%d-img%dx%d" % c for c in CASES])
def test_direct_convolution_shapes(envs, kw, kh, w, h):
    env64, env32 = envs
    psf = _psf(kw, kh)
    profiles = _profiles(w, h)
    y, x = np.mgrid[0:h, 0:w]
    cot = 1.0 + 0.5 * np.sin(x / 7.0) * np.cos(y / 5.0)

    img64, g64, _ = _run(env64, True, w, h, psf, profiles, cot)
    img32, g32, info = _run(env32, False, w, h, psf, profiles, cot)
    _SHAPES.add(info["forward_shape"])
    assert info["fft_models"] == 0

    # forward
    assert abs(img32.sum() - img64.sum()) <= 1e-5 * abs(img64.sum())
    peak = np.abs(img64).max()
    bright = np.abs(img64) > 1e-3 * peak
    assert np.max(np.abs(img32[bright] - img64[bright]) / np.abs(img64[bright])) <= 1e-4

    # adjoint through the magnitude slots: -0.4 ln 10 <c, image of profile i alone>
    for i in (0, 1):
        alone, _, _ = _run(env64, True, w, h, psf, [profiles[i]], cot)
        want = -0.4 * LN10 * float(np.sum(cot * alone))
        assert abs(g64[i, 2] - want) <= 1e-10 * abs(want), (i, g64[i, 2], want)
        assert abs(g32[i, 2] - want) <= 1e-4 * abs(want), (i, g32[i, 2], want)

    # every gradient, FP32 against FP64
    scale = np.abs(g64).max()
    assert np.all(np.abs(g32 - g64) <= 1e-3 * np.abs(g64) + 1e-4 * scale), np.abs(g32 - g64).max() / scale


N_SHAPES = 5


@pytest.mark.parametrize("shape", range(N_SHAPES))
def test_every_block_shape(envs, shape, monkeypatch):
    """Each single-precision block shape (the autotuner may pick any, the
    least-area rule never picks shape 3), forced with PF_CONV_SHAPE, in both directions on
    a ragged image with a 25 x 25 and a 7 x 6 PSF, against the plain FP64
    path as above."""
    env64, env32 = envs
    monkeypatch.setenv("PF_CONV_SHAPE", str(shape))
    w, h = 131, 77
    y, x = np.mgrid[0:h, 0:w]
    cot = 1.0 + 0.5 * np.sin(x / 7.0) * np.cos(y / 5.0)
    for kw, kh in ((25, 25), (7, 6)):
        psf = _psf(kw, kh)
        profiles = _profiles(w, h)
        img64, g64, _ = _run(env64, True, w, h, psf, profiles, cot)
        img32, g32, info = _run(env32, False, w, h, psf, profiles, cot)
        assert info["forward_shape"] == shape and info["adjoint_shape"] == shape
        assert abs(img32.sum() - img64.sum()) <= 1e-5 * abs(img64.sum())
        peak = np.abs(img64).max()
        bright = np.abs(img64) > 1e-3 * peak
        assert np.max(np.abs(img32[bright] - img64[bright]) / np.abs(img64[bright])) <= 1e-4
        scale = np.abs(g64).max()
        assert np.all(np.abs(g32 - g64) <= 1e-3 * np.abs(g64) + 1e-4 * scale), np.abs(g32 - g64).max() / scale


@pytest.mark.parametrize("shape", range(N_SHAPES))
def test_compiled_stride_equals_stride_read_per_model(envs, shape, monkeypatch):
    """The kernels with the PSF row stride compiled in (taken where every
    convolved model's PSF is 13 to 32 wide and rounds up to the same multiple
    of four) give the bits of the kernels that read the stride per model
    (PF_CONV_STRIDE=0), forward and adjoint, with each block shape, for PSF
    widths with every kw mod 4 and the tail pass."""
    env64, env32 = envs
    monkeypatch.setenv("PF_CONV_SHAPE", str(shape))
    w, h = 131, 77
    y, x = np.mgrid[0:h, 0:w]
    cot = 1.0 + 0.5 * np.sin(x / 7.0) * np.cos(y / 5.0)
    for kw, kh in ((13, 9), (18, 18), (23, 6), (25, 25), (32, 11)):
        psf = _psf(kw, kh)
        profiles = _profiles(w, h)
        monkeypatch.delenv("PF_CONV_STRIDE", raising=False)
        img_c, g_c, _ = _run(env32, False, w, h, psf, profiles, cot)
        monkeypatch.setenv("PF_CONV_STRIDE", "0")
        img_r, g_r, _ = _run(env32, False, w, h, psf, profiles, cot)
        assert np.array_equal(img_c, img_r), (kw, kh)
        assert np.array_equal(g_c, g_r), (kw, kh)


def test_block_shapes_covered():
    """The image sizes above select at least four of the five block shapes
    (shape 3 has shape 1's tile, so the least-area rule never picks it)."""
    if len(_SHAPES) == 0:
        pytest.skip("runs after the shape cases")
    assert {0, 1, 2, 4} <= _SHAPES, _SHAPES


def test_large_psf_takes_a_block_shape_that_fits(envs):
    """A 121 x 121 PSF: the least-area block shape's patch does not fit in
    shared memory, a smaller one does and is taken, forward and adjoint; the
    image against the FP64 path, the gradients against the same model's FFT
    convolution."""
    import torch
    import libprofit_gb300 as pg
    import workloads as W
    env64, env32 = envs
    w, h = 256, 256
    psf = W.moffat_psf(121, 4.0, 2.5)
    profiles = _profiles(w, h)

    def run(env, conv, dt):
        m = W.to_model(dict(width=w, height=h, psf=psf, profiles=profiles), env)
        m.set_convolver(conv)
        b = pg.Batch([m], env)
        img = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
        b.forward(img)
        b.check()
        out = img.cpu().numpy().astype(np.float64).reshape(h, w)
        g = None
        if dt == torch.float32:
            b.enable_adjoint()
            y, x = np.mgrid[0:h, 0:w]
            cot = torch.tensor((1.0 + 0.5 * np.sin(x / 7.0) * np.cos(y / 5.0)).ravel(), dtype=dt, device="cuda")
            grad = torch.zeros(len(profiles) * 12, dtype=torch.float64, device="cuda")
            b.backward(img, cotangent=cot, grad=grad)
            b.check()
            g = grad.cpu().numpy()
        return out, g, b.conv_info()

    ref, _, _ = run(env64, "brute", torch.float64)
    img, g, info = run(env32, "brute", torch.float32)
    assert info["fft_models"] == 0
    assert abs(img.sum() - ref.sum()) <= 1e-5 * abs(ref.sum())
    peak = np.abs(ref).max()
    bright = np.abs(ref) > 1e-3 * peak
    assert np.max(np.abs(img[bright] - ref[bright]) / np.abs(ref[bright])) <= 1e-4
    _, gf, _ = run(env32, "fft", torch.float32)
    scale = np.abs(gf).max()
    assert np.all(np.abs(g - gf) <= 1e-4 * np.abs(gf) + 1e-6 * scale)


def test_psf_beyond_direct_takes_fft_automatically(envs):
    """A 181 x 181 PSF fits no direct block shape's shared memory: the
    automatic choice takes the FFT whatever the cost model says; the image
    against the FP64 path (direct) at the FFT's bars."""
    import workloads as W
    env64, env32 = envs
    spec = dict(width=200, height=180, psf=W.moffat_psf(181, 5.0, 2.5), profiles=_profiles(200, 180))
    ref = W.to_model(dict(spec, convolver="brute"), env64).evaluate()
    img = W.to_model(dict(spec, convolver="auto"), env32).evaluate()
    assert abs(img.sum() - ref.sum()) <= 1e-5 * abs(ref.sum())
    peak = np.abs(ref).max()
    assert np.max(np.abs(img - ref)) <= 2e-6 * peak
