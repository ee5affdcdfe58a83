"""Parameter validation and model checks on the host (no GPU needed).

pf_model_output_dims runs the same validation as Model::evaluate (the
profiles' validate() methods, src/*.cpp, and analyze_inputs,
src/model.cpp:186-219) before any device work. Every invalid case must raise
InvalidParameter with the message the oracle restatement gives and, when the
reference compiled here (oracle/_ref), the message the reference itself
throws.
"""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

CASES = [
    ("sersic", dict(axrat=0.0), "axrat <= 0, must have axrat > 0"),
    ("sersic", dict(axrat=1.5), "axrat > 1, must have axrat <= 1"),
    ("moffat", dict(box=-2.0), "box <= -2, must have box > -2"),
    ("sersic", dict(re=0.0), "re <= 0, must have re > 0"),
    ("sersic", dict(nser=-1.0), "nser <= 0, must have nser > 0"),
    ("coresersic", dict(rb=0.0), "rb <= 0, must have rb > 0"),
    ("coresersic", dict(a=0.0), "a <= 0, must have a > 0"),
    ("coresersic", dict(b=2.5), "b > 1.999, must have b < 1.999"),
    ("moffat", dict(fwhm=0.0), "fwhm <= 0, must have fwhm > 0"),
    ("moffat", dict(con=-0.5), "con < 0, must have con >= 0"),
    ("ferrer", dict(rout=0.0), "rout <= 0, must have rout >= 0"),
    ("ferrer", dict(a=-1.0), "a < 0, must have a >= 0"),
    ("ferrer", dict(b=2.5), "b > 2, must have b <= 2"),
    ("king", dict(rc=0.0), "rc <= 0, must have rc > 0"),
    ("king", dict(rt=-1.0), "rt <= 0, must have rt > 0"),
    ("king", dict(a=-1.0), "a < 0, must have a >=0"),
    ("brokenexp", dict(h1=0.0), "h1 <= 0, must have h1 > 0"),
    ("brokenexp", dict(h2=0.0), "h2 <= 0, must have h2 > 0"),
    ("brokenexp", dict(rb=0.0), "rb <= 0, must have rb > 0"),
]


def _gpu_message(width, height, profiles, psf=None, mask=None, adjust_mask=True):
    import libprofit_gb300 as pg
    m = pg.Model(width, height)
    if psf is not None:
        m.set_psf(psf)
    if mask is not None:
        m.set_mask(mask)
        m.set_adjust_mask(adjust_mask)
    for kind, params in profiles:
        p = m.add_profile(kind)
        for k, v in params.items():
            p.parameter(k, bool(v) if k == "convolve" else float(v))
    with pytest.raises(pg.InvalidParameter) as e:
        m.output_dims()
    return str(e.value)


def _ref_available():
    return os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libprofit_ref.so"))


@pytest.mark.parametrize("kind,params,msg", CASES, ids=["%s-%s" % (c[0], list(c[1])[0]) for c in CASES])
def test_profile_validation_messages(oracle_lib, kind, params, msg):
    O = oracle_lib
    got = _gpu_message(10, 10, [(kind, params)])
    assert got == msg
    with pytest.raises(O.OracleError) as e:
        O.evaluate(O.Case(10, 10, [(kind, params)]))
    assert str(e.value) == msg
    if _ref_available():
        with pytest.raises(O.OracleError) as e:
            O.evaluate_reference(O.Case(10, 10, [(kind, params)]))
        assert str(e.value) == msg


def test_model_checks(oracle_lib):
    O = oracle_lib
    assert _gpu_message(0, 10, [("sersic", {})]) == "Model's requested dimensions are 0"
    assert _gpu_message(10, 10, [("sersic", dict(convolve=True))]) == \
        "No psf provided but profile(s) requested convolution"
    assert _gpu_message(10, 10, [("psf", {})]) == "No psf present in the model, cannot produce a psf profile"
    mask = np.ones((9, 10), np.uint8)
    assert _gpu_message(10, 10, [("sersic", {})], mask=mask) == "Mask dimensions != model dimensions"
    with pytest.raises(O.OracleError, match="Mask dimensions != model dimensions"):
        O.evaluate(O.Case(10, 10, [("sersic", {})], mask=mask))


def test_device_buffer_sizes_checked_on_the_host():
    """The C ABI takes raw device pointers; the Python Batch methods refuse a
    buffer with too few elements or another element size before any launch
    (a parameter vector of one row per model instead of one per profile would
    otherwise be read past its end)."""
    import libprofit_gb300 as pg

    class Buf:
        def __init__(self, n, size):
            self.n, self.size = n, size

        def numel(self):
            return self.n

        def element_size(self):
            return self.size

    pg._need(Buf(384, 8), 384, 8, "params")
    pg._need(Buf(400, 8), 384, 8, "params")
    pg._need(None, 384, 8, "params")
    with pytest.raises(pg.InvalidParameter, match="params: 384 elements of 8 bytes needed, the buffer has 192 of 8"):
        pg._need(Buf(192, 8), 384, 8, "params")
    with pytest.raises(pg.InvalidParameter, match="images"):
        pg._need(Buf(1000, 8), 1000, 4, "images")


def test_batch_refuses_host_foreign_and_strided_buffers():
    """A tensor in host memory, on another device than the environment's, or
    not contiguous is refused: the C ABI would read or write its data pointer
    as one dense array on the environment's device."""
    import torch
    import libprofit_gb300 as pg

    class Dev:
        def __init__(self, index):
            self.index = index

    class Buf:
        def __init__(self, n, cuda=True, index=0, contiguous=True):
            self.n, self.is_cuda, self.device, self.c = n, cuda, Dev(index), contiguous

        def numel(self):
            return self.n

        def element_size(self):
            return 8

        def is_contiguous(self):
            return self.c

    pg._need(Buf(16), 16, 8, "grad", 0)
    with pytest.raises(pg.InvalidParameter, match="grad: a device .* host memory"):
        pg._need(torch.zeros(16, dtype=torch.float64), 16, 8, "grad", 0)
    with pytest.raises(pg.InvalidParameter, match="chi2: the buffer is on device 1, the environment on device 0"):
        pg._need(Buf(16, index=1), 16, 8, "chi2", 0)
    with pytest.raises(pg.InvalidParameter, match="flux: the buffer must be contiguous"):
        pg._need(Buf(16, contiguous=False), 16, 8, "flux", 0)


def test_uncropped_fft_dimensions_and_offset(oracle_lib):
    """The dimensions and offset of Model::evaluate with crop = false and the
    FFT convolver (pf_model_output_dims / pf_model_output_offset, no GPU
    needed) equal those of the oracle's restatement of the reference's
    arithmetic (src/model.cpp:288-306, src/convolve.cpp:263-281)."""
    import workloads as W
    import libprofit_gb300 as pg
    for w, h, k in [(40, 40, 9), (41, 37, 8), (60, 30, 10), (33, 30, 15), (12, 12, 9), (30, 34, 7), (64, 20, 16)]:
        profs = [("sersic", dict(xcen=w / 2, ycen=h / 2, mag=15.0, re=3.0, convolve=True))]
        spec = dict(width=w, height=h, psf=W.moffat_psf(k, 2.5, 2.5), profiles=profs)
        m = W.to_model(spec)
        m.set_convolver("fft")
        m.set_crop(False)
        ref, ref_off = oracle_lib.evaluate_uncropped_fft(oracle_lib.Case(w, h, profs, psf=spec["psf"]))
        assert m.output_dims() == (ref.shape[1], ref.shape[0])
        assert m.output_offset() == ref_off


def test_no_user_profile_in_the_default_build():
    """The default library has no user-defined profile compiled in: the C ABI
    says so, and its name is unknown to Model.add_profile."""
    import ctypes
    import libprofit_gb300 as pg
    from libprofit_gb300 import _ffi
    name = ctypes.c_char_p()
    assert _ffi.load().pf_user_profile_info(ctypes.byref(name), None, None, None) == _ffi.PF_ERR_UNSUPPORTED
    with pytest.raises(pg.InvalidParameter, match="Unknown profile name: usermoffat"):
        pg.Model(10, 10).add_profile("usermoffat")
