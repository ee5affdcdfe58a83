"""Model::set_crop and the mask dimension checks (GPU).

The reference's own case (tests/test_model.h:343-385): a 20 x 20 model with a
convolved null profile and a 2 x 2 PSF, finesampling 1 and 2, brute-force
convolution: the uncropped image has the cropped dimensions, offset (0, 0),
and equals the cropped image. This backend's direct convolutions behave the
same (Convolver::padding is empty for them, src/convolve.cpp:50-53), so do
the automatic and CUDA convolvers. The FFT convolver with crop = false keeps
its uncropped frame less the PSF padding (src/model.cpp:288-306,
src/convolve.cpp:263-312): image, dimensions and offset against the oracle's
numpy restatement of that arithmetic (the compiled reference has no FFTW
here), to 1e-12 of the peak (FFT rounding is absolute); the cases it does not
cover are refused. Masks whose dimensions do not match raise the reference's
messages (src/model.cpp:198-201, 277-283).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    return pg.get_cuda_environment(0, use_double=True)


def _model(pg, env, fs, convolver, profile="null"):
    m = pg.Model(20, 20)
    m.set_cuda_env(env)
    m.set_convolver(convolver)
    m.set_psf(np.ones((2, 2)))
    m.set_finesampling(fs)
    p = m.add_profile(profile)
    p.parameter("convolve", True)
    if profile == "sersic":
        p.parameter("xcen", 9.7)
        p.parameter("ycen", 10.4)
        p.parameter("re", 4.0)
    return m


@pytest.mark.parametrize("fs", [1, 2])
@pytest.mark.parametrize("convolver", ["brute", "auto", "cuda"])
@pytest.mark.parametrize("profile", ["null", "sersic"])
def test_no_crop_direct_convolution(env, fs, convolver, profile):
    import libprofit_gb300 as pg
    m = _model(pg, env, fs, convolver, profile)
    original = m.evaluate()
    assert original.shape == (20 * fs, 20 * fs)
    m.set_crop(False)
    uncropped, offset = m.evaluate_with_offset()
    assert uncropped.shape == (20 * fs, 20 * fs)
    assert offset == (0, 0)
    assert np.array_equal(original, uncropped[offset[1]:offset[1] + 20 * fs, offset[0]:offset[0] + 20 * fs])


# (width, height, PSF side, with a non-convolved profile): odd and even
# PSFs, square, wide and slightly tall images, a small image
FFT_CASES = [(40, 40, 9, True), (41, 37, 8, True), (60, 30, 10, False), (33, 30, 15, True), (12, 12, 9, True),
             (30, 34, 7, True)]


def _fft_spec(w, h, k, direct):
    import workloads as W
    profs = [("sersic", dict(xcen=w / 2 + 0.3, ycen=h / 2 - 0.2, mag=15.0, re=4.0, nser=2.2, ang=20.0, axrat=0.7,
                             convolve=True)),
             ("sky", dict(bg=0.01))]
    if direct:
        profs.append(("sersic", dict(xcen=w / 3, ycen=h / 3, mag=17.0, re=2.0, nser=1.0, ang=60.0, axrat=0.5)))
    return dict(width=w, height=h, psf=W.moffat_psf(k, 2.5, 2.5), profiles=profs)


@pytest.mark.parametrize("w,h,k,direct", FFT_CASES)
def test_no_crop_fft_uncropped_frame(env, oracle_lib, w, h, k, direct):
    import workloads as W
    spec = _fft_spec(w, h, k, direct)
    m = W.to_model(spec, env)
    m.set_convolver("fft")
    cropped = m.evaluate()
    m.set_crop(False)
    img, offset = m.evaluate_with_offset()
    ref, ref_off = oracle_lib.evaluate_uncropped_fft(oracle_lib.Case(w, h, spec["profiles"], psf=spec["psf"]))
    assert img.shape == ref.shape
    assert offset == ref_off
    peak = np.abs(ref).max()
    assert np.abs(img - ref).max() <= 1e-12 * peak
    # the requested area at the offset is the cropped image
    sub = img[offset[1]:offset[1] + h, offset[0]:offset[0] + w]
    assert np.abs(sub - cropped).max() <= 1e-12 * peak


def test_no_crop_fft_refusals(env):
    import libprofit_gb300 as pg
    import workloads as W
    spec = _fft_spec(30, 50, 7, False)  # the reference's frame wraps around
    m = W.to_model(spec, env)
    m.set_convolver("fft")
    m.set_crop(False)
    with pytest.raises(pg.Unsupported, match="wraps around"):
        m.evaluate()
    spec = _fft_spec(40, 40, 9, False)
    m = W.to_model(spec, env)
    m.set_convolver("fft")
    m.set_crop(False)
    m.set_finesampling(2)
    m.set_return_finesampled(False)
    with pytest.raises(pg.Unsupported, match="SUM-downsampled"):
        m.evaluate()
    m = W.to_model(spec, env)
    m.set_convolver("fft")
    m.set_crop(False)
    mask = np.zeros((40, 40), np.uint8)
    mask[5:30, 8:33] = 1
    m.set_mask(mask)
    with pytest.raises(pg.Unsupported, match="adjustable calculation mask"):
        m.evaluate()
    env32 = pg.get_cuda_environment(0, use_double=False)
    m = W.to_model(spec, env32)
    m.set_convolver("fft")
    m.set_crop(False)
    with pytest.raises(pg.Unsupported, match="double precision"):
        m.evaluate()


def test_mask_dimension_checks(env):
    import libprofit_gb300 as pg
    m = _model(pg, env, 1, "brute", "sersic")
    m.set_mask(np.ones((19, 20), np.uint8))
    with pytest.raises(pg.InvalidParameter, match="Mask dimensions != model dimensions"):
        m.evaluate()
    m.set_adjust_mask(False)
    # larger than the model: padded drawing area (20 + 2 * 1) expected
    m.set_mask(np.ones((23, 23), np.uint8))
    with pytest.raises(pg.InvalidParameter, match=r"Mask dimensions != drawing dimensions: \[23, 23\] != \[22, 22\]"):
        m.evaluate()
    m.set_mask(np.ones((22, 22), np.uint8))
    assert m.evaluate().shape == (20, 20)
    m.set_mask(np.ones((20, 20), np.uint8))  # the model's size: no padding
    assert m.evaluate().shape == (20, 20)
