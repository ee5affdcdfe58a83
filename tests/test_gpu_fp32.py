"""Single-precision batched path against the reference (GPU).

Bar (per pixel and total flux against the FP64 reference images):
  * relative error <= 1e-4 for every pixel brighter than FLOOR x the image's
    peak, where FLOOR = 1e-9 (fainter pixels are checked in absolute terms:
    |err| <= 1e-4 * FLOOR * peak);
  * total flux relative error <= 1e-5;
  * the subsampling tree (per-pixel depth map and per-level counts) equals the
    oracle's: every FP32 decision near its threshold is re-taken in FP64.
"""
import numpy as np
import pytest

from tests.golden.load import load, to_case
from tests.helpers import product_model

pytestmark = pytest.mark.gpu

GOLDEN = load()
PIX_TOL = 1e-4
FLUX_TOL = 1e-5
FLOOR = 1e-9
RADIAL = ("sersic", "coresersic", "moffat", "ferrer", "king", "brokenexp")


@pytest.fixture(scope="module")
def env32():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    return pg.get_cuda_environment(0, use_double=False)


def check_fp32(img, ref, name=""):
    assert img.shape == ref.shape
    peak = np.abs(ref).max()
    if peak == 0:
        assert np.all(img == 0)
        return
    bright = np.abs(ref) > FLOOR * peak
    rel = np.abs(img[bright] - ref[bright]) / np.abs(ref[bright])
    faint_err = np.abs(img[~bright] - ref[~bright])
    assert rel.max() <= PIX_TOL, "%s: max rel err %.3g" % (name, rel.max())
    assert faint_err.size == 0 or faint_err.max() <= PIX_TOL * FLOOR * peak
    flux_rel = abs(img.sum() - ref.sum()) / abs(ref.sum())
    assert flux_rel <= FLUX_TOL, "%s: flux rel err %.3g" % (name, flux_rel)


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_fp32_matches_reference(env32, name):
    entry = GOLDEN[name]
    img = product_model(entry["spec"], entry["psf"], env32).evaluate()
    check_fp32(img, entry["image"], name)


def _radial_single(name):
    profs = GOLDEN[name]["spec"]["profiles"]
    return len(profs) == 1 and profs[0][0] in RADIAL


@pytest.mark.parametrize("name", sorted(n for n in GOLDEN if _radial_single(n)))
def test_fp32_tree_equals_oracle(env32, oracle_lib, name):
    import torch
    import libprofit_gb300 as pg
    O = oracle_lib
    entry = GOLDEN[name]
    m = product_model(entry["spec"], entry["psf"], env32)
    b = pg.Batch([m], env32)
    b.record_depth(True)
    out = torch.zeros(b.total_pixels, dtype=torch.float32, device="cuda")
    b.forward(out)
    b.check()
    (depth, counts), = b.depth()
    _, odepth, ocounts = O.evaluate(to_case(O, entry), want_depth=True)
    assert np.array_equal(depth, odepth[0]), "depth differs at %d pixels" % int((depth != odepth[0]).sum())
    assert np.array_equal(counts[:16], ocounts[0][:16])


def test_fp32_batch_equals_single():
    """Models packed in one batch render as they do alone, bit for bit, in an
    environment without timed choices (PF_ENV_NO_AUTOTUNE: the timed split
    of the subsampling trees may add a multi-profile pixel's values in
    another order, which can move its last bit)."""
    import torch
    import libprofit_gb300 as pg
    env32 = pg.CUDAEnv(0, use_double=False, autotune=False)
    names = ["cfg1_sersic_brute", "king_rotated", "mixed_conv_sky_psf", "finesampled", "brokenexp_shaped"]
    models = [product_model(GOLDEN[n]["spec"], GOLDEN[n]["psf"], env32) for n in names]
    b = pg.Batch(models, env32)
    out = torch.zeros(b.total_pixels, dtype=torch.float32, device="cuda")
    flux = torch.zeros(len(models), dtype=torch.float64, device="cuda")
    b.forward(out, flux)
    b.check()
    o = out.cpu().numpy()
    for i, n in enumerate(names):
        w, h = b.dims[i]
        img = o[b.offsets[i]:b.offsets[i + 1]].reshape(h, w)
        assert np.array_equal(img.astype(np.float64), models[i].evaluate())
        check_fp32(img.astype(np.float64), GOLDEN[n]["image"], n)
        assert abs(flux[i].item() - img.astype(np.float64).sum()) <= 1e-6 * abs(img.sum())


def _forward32(m, env):
    import torch
    import libprofit_gb300 as pg
    b = pg.Batch([m], env)
    b.record_depth(True)
    out = torch.zeros(b.total_pixels, dtype=torch.float32, device="cuda")
    b.forward(out)
    b.check()
    maps = b.depth()
    return out.cpu().numpy(), [d for d, _ in maps], np.array([c for _, c in maps]), b.split_info()


def test_fp32_split_equals_walk(env32, monkeypatch):
    """The subsampling trees split off to other warps (PF_SPLIT=1) or walked
    where met (PF_SPLIT=0; the batch otherwise times both): the same depth
    maps and per-level counts, the same image bits for one-profile models,
    and several-profile pixels within the last bit (addition order)."""
    used = 0
    for name in sorted(GOLDEN):
        entry = GOLDEN[name]
        runs = []
        for mode in ("1", "0"):
            monkeypatch.setenv("PF_SPLIT", mode)
            runs.append(_forward32(product_model(entry["spec"], entry["psf"], env32), env32))
        (a, da, ca, info), (w, dw, cw, winfo) = runs
        assert winfo["boxes"] == 0
        used += info["boxes"]
        assert len(da) == len(dw) and all(np.array_equal(x, y) for x, y in zip(da, dw)), name
        assert np.array_equal(ca, cw), name
        if len(entry["spec"]["profiles"]) == 1:
            assert np.array_equal(a, w), name
        else:
            np.testing.assert_allclose(a, w, rtol=1e-6, atol=0, err_msg=name)
    assert used > 0
