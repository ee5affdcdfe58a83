"""Plain FP64 CUDA path against the reference (GPU).

Every golden image of tests/golden (rendered by the unmodified libprofit)
must be reproduced to <= 1e-10 relative per pixel, pixels that are exactly 0
in the reference must be exactly 0, the per-pixel subsampling depth maps must
equal the oracle restatement's bit for bit, and the per-level subsample_pixel
counts must equal the reference's PROFIT_DEBUG n_integrations
(src/radial.cpp:71-79).
"""
import numpy as np
import pytest

from tests.golden.load import load, to_case
from tests.helpers import product_model

pytestmark = pytest.mark.gpu

GOLDEN = load()
TOL = 1e-10  # relative, per pixel
RADIAL = ("sersic", "coresersic", "moffat", "ferrer", "king", "brokenexp")


@pytest.fixture(scope="module")
def env():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    return pg.get_cuda_environment(0, use_double=True)


def check_image(img, ref):
    assert img.shape == ref.shape
    zero = ref == 0
    assert np.array_equal(img[zero], ref[zero]), "pixels that are 0 in the reference must be 0"
    nz = ~zero
    rel = np.abs(img[nz] - ref[nz]) / np.abs(ref[nz])
    assert rel.size == 0 or rel.max() <= TOL, "max rel err %.3g" % rel.max()


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_fp64_matches_reference(env, name):
    entry = GOLDEN[name]
    img = product_model(entry["spec"], entry["psf"], env).evaluate()
    check_image(img, entry["image"])


def _radial_single(name):
    profs = GOLDEN[name]["spec"]["profiles"]
    return len(profs) == 1 and profs[0][0] in RADIAL


@pytest.mark.parametrize("name", sorted(n for n in GOLDEN if _radial_single(n)))
def test_depth_map_and_counts(env, oracle_lib, name):
    import torch
    import libprofit_gb300 as pg
    O = oracle_lib
    entry = GOLDEN[name]
    m = product_model(entry["spec"], entry["psf"], env)
    b = pg.Batch([m], env)
    b.record_depth(True)
    out = torch.zeros(b.total_pixels, dtype=torch.float64, device="cuda")
    b.forward(out)
    b.check()
    (depth, counts), = b.depth()
    _, odepth, ocounts = O.evaluate(to_case(O, entry), want_depth=True)
    assert np.array_equal(depth, odepth[0]), "depth map differs at %d pixels" % int((depth != odepth[0]).sum())
    assert np.array_equal(counts[:16], entry["counts"][0][:16])
    assert np.array_equal(counts[:16], ocounts[0][:16])
    check_image(out.cpu().numpy().reshape(entry["image"].shape), entry["image"])


def test_batch_equals_single_models(env):
    """Models packed in one batch render exactly as they do alone."""
    import torch
    import libprofit_gb300 as pg
    names = ["cfg1_sersic_brute", "king_rotated", "mixed_conv_sky_psf", "finesampled_downsampled",
             "coresersic_shaped", "sersic_scale_magzero"]
    models = [product_model(GOLDEN[n]["spec"], GOLDEN[n]["psf"], env) for n in names]
    b = pg.Batch(models, env)
    out = torch.zeros(b.total_pixels, dtype=torch.float64, device="cuda")
    flux = torch.zeros(len(models), dtype=torch.float64, device="cuda")
    b.forward(out, flux)
    b.check()
    o = out.cpu().numpy()
    for i, n in enumerate(names):
        w, h = b.dims[i]
        img = o[b.offsets[i]:b.offsets[i + 1]].reshape(h, w)
        assert np.array_equal(img, models[i].evaluate())
        check_image(img, GOLDEN[n]["image"])
        assert abs(flux[i].item() - img.sum()) <= 1e-12 * abs(img.sum())


def test_repeatable_and_param_update(env):
    """Two forwards give identical bits; set_params re-derives every constant
    (the adjust step is applied to the descriptor's values each time)."""
    import torch
    import libprofit_gb300 as pg
    entry = GOLDEN["sersic_shaped"]
    m = product_model(entry["spec"], entry["psf"], env)
    b = pg.Batch([m], env)
    a = torch.zeros(b.total_pixels, dtype=torch.float64, device="cuda")
    c = torch.zeros_like(a)
    b.forward(a)
    b.forward(c)
    b.check()
    assert torch.equal(a, c)
    par = np.array([m.profiles[0].desc.par[i] for i in range(12)])
    par2 = par.copy()
    par2[7] = 3.7   # nser
    par2[0] += 0.25  # xcen
    b.set_params(par2)
    b.forward(c)
    b.check()
    m.profiles[0].parameter("nser", 3.7)
    m.profiles[0].parameter("xcen", par2[0])
    assert np.array_equal(c.cpu().numpy().reshape(entry["image"].shape), m.evaluate())
    b.set_params_dev(torch.tensor(par, dtype=torch.float64, device="cuda"))
    b.forward(c)
    b.check()
    assert torch.equal(a, c)


def test_convolver_matches_reference_brute(env, oracle_lib):
    """pf_convolve vs the associative brute-force convolver, incl. a mask and a
    kernel larger than the image (tests/test_convolver.h:112-191)."""
    import libprofit_gb300 as pg
    O = oracle_lib
    rng = np.random.default_rng(11)
    conv = pg.create_convolver("cuda", env)
    for (h, w), (kh, kw) in [((100, 100), (25, 25)), ((101, 99), (24, 25)), ((37, 64), (15, 16))]:
        src, krn = rng.random((h, w)), rng.random((kh, kw))
        ref = O.convolve_brute(src, krn)
        np.testing.assert_allclose(conv.convolve(src, krn), ref, rtol=1e-13, atol=0)
        mask = rng.random((h, w)) > 0.3
        refm = O.convolve_brute(src, krn, mask=mask)
        got = conv.convolve(src, krn, mask=mask)
        assert np.all(got[~mask] == 0)
        np.testing.assert_allclose(got, refm, rtol=1e-13, atol=0)
    # kernel larger than the image: extended to max(src, krn), convolved, cropped back
    src, krn = rng.random((10, 10)), rng.random((15, 15))
    ext = np.zeros((15, 15))
    ext[:10, :10] = src
    ref = O.convolve_brute(ext, krn)[:10, :10]
    np.testing.assert_allclose(conv.convolve(src, krn), ref, rtol=1e-13, atol=0)
    # the extension's height repeats the width maximum; one below the image's
    # height is refused, as Surface::extend refuses it
    with pytest.raises(pg.InvalidParameter):
        conv.convolve(rng.random((40, 10)), rng.random((15, 15)))


@pytest.mark.parametrize("name", sorted(n for n in GOLDEN if _radial_single(n))[::4])
def test_model_profile_integrations(env, name):
    """Model.get_profile_integrations against the reference's PROFIT_DEBUG
    n_integrations (src/model.cpp:370-381): {level: count} of the levels the
    reference counted, keyed by the profile's name."""
    entry = GOLDEN[name]
    m = product_model(entry["spec"], entry["psf"], env)
    got = m.get_profile_integrations()
    kind = entry["spec"]["profiles"][0][0]
    want = {lvl: int(c) for lvl, c in enumerate(entry["counts"][0][:16]) if c > 0}
    assert got == {kind: want}


def _forward_depth(m, env):
    import torch
    import libprofit_gb300 as pg
    b = pg.Batch([m], env)
    b.record_depth(True)
    out = torch.zeros(b.total_pixels, dtype=torch.float64, device="cuda")
    b.forward(out)
    b.check()
    maps = b.depth()
    depth = [d for d, _ in maps]
    counts = np.array([c for _, c in maps])
    return out.cpu().numpy(), depth, counts, b.split_info()


@pytest.mark.parametrize("pool_boxes", [None, "40"])
def test_level_pool_equals_tile_walk(env, pool_boxes, monkeypatch):
    """The subsampling trees evaluated level by level over the whole GPU give
    the depth-first walk's results: the same depth maps and per-level counts,
    and the same image bits for one-profile models (each box's sum is formed
    in the walk's order; a pixel's subsampled profiles are added after its
    other profiles, so several-profile pixels may differ by rounding). With
    a pool of 40 boxes most trees find no room and are walked in place, at
    level 0 by the tile's warp or deeper by the level kernel's."""
    import libprofit_gb300 as pg
    if pool_boxes:
        monkeypatch.setenv("PF_LEVEL_POOL_BOXES", pool_boxes)
    walk = pg.CUDAEnv(0, use_double=True, split=False)
    roots = refused = 0
    for name in sorted(GOLDEN):
        entry = GOLDEN[name]
        a, da, ca, info = _forward_depth(product_model(entry["spec"], entry["psf"], env), env)
        w, dw, cw, winfo = _forward_depth(product_model(entry["spec"], entry["psf"], walk), walk)
        assert winfo == {"boxes": 0, "roots": 0, "pixels": 0, "refused": 0}
        roots += info["roots"]
        refused += info["refused"]
        assert len(da) == len(dw) and all(np.array_equal(x, y) for x, y in zip(da, dw)), name
        assert np.array_equal(ca, cw), name
        if len(entry["spec"]["profiles"]) == 1:
            assert np.array_equal(a, w), name
        else:
            np.testing.assert_allclose(a, w, rtol=1e-14, atol=0, err_msg=name)
    assert roots > 0
    assert (refused > 0) == bool(pool_boxes)
