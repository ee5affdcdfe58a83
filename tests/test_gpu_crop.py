"""Model::set_crop and the mask dimension checks (GPU).

The reference's own case (tests/test_model.h:343-385): a 20 x 20 model with a
convolved null profile and a 2 x 2 PSF, finesampling 1 and 2, brute-force
convolution: the uncropped image has the cropped dimensions, offset (0, 0),
and equals the cropped image. This backend's direct convolutions behave the
same (Convolver::padding is empty for them, src/convolve.cpp:50-53), so do
the automatic and CUDA convolvers; the FFT convolver with crop = false is
refused. Masks whose dimensions do not match raise the reference's messages
(src/model.cpp:198-201, 277-283).
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


def test_no_crop_fft_refused(env):
    import libprofit_gb300 as pg
    m = _model(pg, env, 1, "fft", "sersic")
    m.evaluate()
    m.set_crop(False)
    with pytest.raises(pg.Unsupported):
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
