"""The drop-in path, Model::evaluate one model at a time (GPU).

A fitting loop calls Model::evaluate over and over on the same model with new
parameter values (src/model.cpp:259-320; profit-cli's -i loop,
src/profit-cli.cpp:390-412). The environment keeps the previous call's device
state and reuses it while only parameter values change:
  * every call gives bit for bit the image a fresh environment gives;
  * after the first call, repeated calls leave the device's free memory
    unchanged (nothing allocated, nothing freed);
  * a change of dimensions, profiles, PSF or mask rebuilds the state and
    still gives the fresh result;
  * invalid values give the reference's message, and a later valid call works;
  * pf_convolve's scratch is kept the same way, and crop = false returns the
    same image at offset (0, 0), as the reference's direct convolvers do.
"""
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _model(pg, env, params, psf, size=100, mask=None):
    m = pg.Model(size, size)
    m.set_psf(psf)
    if mask is not None:
        m.set_mask(mask)
    m.set_cuda_env(env)
    p = m.add_profile("sersic")
    for k, v in params.items():
        p.parameter(k, v)
    p.parameter("convolve", True)
    s = m.add_profile("sky")
    s.parameter("bg", 1e-3)
    return m


def _params(rng):
    return dict(xcen=50.3 + rng.uniform(-2, 2), ycen=50.7 + rng.uniform(-2, 2), mag=15.0 + rng.uniform(-.5, .5),
                re=8.0 * (1 + 0.1 * rng.uniform(-1, 1)), nser=4.0 * (1 + 0.1 * rng.uniform(-1, 1)),
                ang=30.0 + rng.uniform(-10, 10), axrat=0.6 + rng.uniform(-0.1, 0.1), box=0.0)


@pytest.mark.parametrize("use_double", [True, False])
def test_repeated_evaluate_reuses_state(use_double):
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    psf = W.moffat_psf(15, 3.0, 2.5)
    env = pg.get_cuda_environment(0, use_double=use_double)
    rng = np.random.default_rng(7)
    _model(pg, env, _params(rng), psf).evaluate()  # builds the state
    for _ in range(20):
        par = _params(rng)
        got = _model(pg, env, par, psf).evaluate()
        fresh_env = pg.get_cuda_environment(0, use_double=use_double)
        want = _model(pg, fresh_env, par, psf).evaluate()
        fresh_env.close()
        np.testing.assert_array_equal(got, want)
    # a fitting loop's calls allocate nothing
    gc.collect()  # earlier objects freed now, not during the measurement
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(20):
        _model(pg, env, _params(rng), psf).evaluate()
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0


def test_layout_changes_rebuild():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    env = pg.get_cuda_environment(0, use_double=True)
    rng = np.random.default_rng(8)
    psf15, psf9 = W.moffat_psf(15, 3.0, 2.5), W.moffat_psf(9, 2.0, 3.0)
    mask = np.zeros((100, 100), dtype=np.uint8)
    mask[20:80, 30:90] = 1
    for kw in [dict(psf=psf15), dict(psf=psf9), dict(psf=psf15, size=80), dict(psf=psf15, mask=mask),
               dict(psf=psf15 * 2.0), dict(psf=psf15)]:
        par = _params(rng)
        got = _model(pg, env, par, **kw).evaluate()
        fresh = pg.get_cuda_environment(0, use_double=True)
        want = _model(pg, fresh, par, **kw).evaluate()
        fresh.close()
        np.testing.assert_array_equal(got, want)


def test_invalid_values_on_reused_state():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    psf = W.moffat_psf(15, 3.0, 2.5)
    env = pg.get_cuda_environment(0, use_double=True)
    rng = np.random.default_rng(9)
    par = _params(rng)
    first = _model(pg, env, par, psf).evaluate()
    for k, v, msg in [("axrat", 0.0, "axrat <= 0, must have axrat > 0"), ("nser", -1.0, "nser <= 0, must have nser > 0"),
                      ("re", 0.0, "re <= 0, must have re > 0")]:
        with pytest.raises(pg.InvalidParameter, match="^%s$" % msg):
            _model(pg, env, dict(par, **{k: v}), psf).evaluate()
    np.testing.assert_array_equal(_model(pg, env, par, psf).evaluate(), first)


def test_convolve_scratch_and_crop():
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    env = pg.get_cuda_environment(0, use_double=True)
    conv = pg.create_convolver("cuda", env)
    rng = np.random.default_rng(10)
    src, krn = rng.random((300, 280)), rng.random((25, 25))
    want = conv.convolve(src, krn)
    gc.collect()  # earlier objects freed now, not during the measurement
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(0)[0]
    for _ in range(20):
        np.testing.assert_array_equal(conv.convolve(src, krn), want)
        small = rng.random((10, 12))
        conv.convolve(small, krn)  # extended to the kernel's size, cropped back
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(0)[0] == free0
    off = [7, 7]
    got = conv.convolve(src, krn, crop=False, offset_out=off)
    np.testing.assert_array_equal(got, want)
    assert off == [0, 0]


def test_get_stats():
    """Model::get_stats (src/model.cpp:362-368) in a profiling environment:
    one entry per profile name (a later profile of the same name replacing an
    earlier one, as in the reference's map), the last evaluation's pass
    times, and the profile's subsample_pixel calls per level, which equal
    get_profile_integrations' (the reference's PROFIT_DEBUG counts)."""
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    psf = W.moffat_psf(15, 3.0, 2.5)
    env = pg.get_cuda_environment(0, use_double=True, profile=True)
    m = _model(pg, env, _params(np.random.default_rng(11)), psf)
    assert m.get_stats() == {}  # nothing evaluated yet
    m.evaluate()
    st = m.get_stats()
    assert set(st) == {"sersic", "sky"}
    s = st["sersic"]
    assert s["pass_evaluation_ms"] > 0 and s["total_ms"] > 0 and s["evaluations"] > 0
    assert s["integrations"] == {k: v for k, v in m.get_profile_integrations()["sersic"].items() if v}
    plain = pg.get_cuda_environment(0, use_double=True)
    m.set_cuda_env(plain)
    m.evaluate()
    assert m.get_stats() == {}
