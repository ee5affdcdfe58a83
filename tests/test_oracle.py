"""The oracle restatement is pinned against the unmodified reference.

Golden images come from libprofit itself (tests/golden/make_golden.py runs the
reference sources through profit::Model). The restatement must reproduce them
bit for bit, except where only the order of a convolution's partial sums
differs (the reference's row dot products, include/profit/dot_product.h), for
which 1e-13 relative is allowed. The per-level subsampling counts must equal
the reference's PROFIT_DEBUG n_integrations (src/radial.cpp:71-79).
"""
import numpy as np
import pytest

from tests.golden.load import load, to_case

GOLDEN = load()


@pytest.mark.parametrize("name", sorted(GOLDEN))
def test_restatement_matches_reference(oracle_lib, name):
    O = oracle_lib
    entry = GOLDEN[name]
    img, _, counts = O.evaluate(to_case(O, entry), threads=1)
    ref = entry["image"]
    assert img.shape == ref.shape
    if any(p[1].get("convolve") for p in entry["spec"]["profiles"]):
        np.testing.assert_allclose(img, ref, rtol=1e-13, atol=1e-300)
    else:
        assert np.array_equal(img, ref)
    radial = [i for i, p in enumerate(entry["spec"]["profiles"])
              if p[0] in ("sersic", "coresersic", "moffat", "ferrer", "king", "brokenexp")]
    kinds = [entry["spec"]["profiles"][i][0] for i in radial]
    if len(radial) == 1 or len(set(kinds)) == len(kinds):
        for i in radial:
            assert np.array_equal(counts[i], entry["counts"][i])


def test_known_answer_psf(oracle_lib):
    # tests/test_psf.h:38-50: a 2x2 uniform PSF at (2,2), mag 0 -> 0.25 in a 2x2 block
    img = GOLDEN["psf_known_answer"]["image"]
    expected = np.zeros((10, 10))
    expected[1:3, 1:3] = 0.25
    np.testing.assert_allclose(img, expected, rtol=1e-9, atol=0)


def test_known_answer_sky(oracle_lib):
    # tests/test_sky.h:37-48
    assert np.all(GOLDEN["sky_known_answer"]["image"] == 1.0)


def test_openmp_equality(oracle_lib):
    # tests/test_radial.h:46-59: threads must not change a single bit
    O = oracle_lib
    for name in ("sersic_default", "coresersic_boxy", "king_rotated", "cfg1_sersic_brute"):
        case = to_case(O, GOLDEN[name])
        a, _, _ = O.evaluate(case, threads=1)
        b, _, _ = O.evaluate(case, threads=4)
        assert np.array_equal(a, b)


def test_profile_addition(oracle_lib):
    # tests/test_model.h:204-229: single-profile models add up to the joint model
    O = oracle_lib
    spec = GOLDEN["addition_three_sersics"]["spec"]
    total = np.zeros((100, 100))
    for p in spec["profiles"]:
        img, _, _ = O.evaluate(O.Case(100, 100, [p]))
        total = total + img
    np.testing.assert_allclose(total, GOLDEN["addition_three_sersics"]["image"], rtol=1e-9)


def test_fft_math_equals_brute(oracle_lib):
    # tests/test_fft.h:93-139: FFT vs brute convolution agree
    O = oracle_lib
    rng = np.random.default_rng(7)
    for (h, w), (kh, kw) in [((99, 99), (25, 25)), ((100, 100), (26, 26)), ((100, 99), (25, 26))]:
        src = rng.random((h, w))
        krn = rng.random((kh, kw))
        a = O.convolve_brute(src, krn)
        b = O.fft_convolve_reference_math(src, krn)
        np.testing.assert_allclose(b, a, rtol=1e-9, atol=1e-12 * np.abs(a).max())


def test_validation_errors(oracle_lib):
    O = oracle_lib
    with pytest.raises(O.OracleError, match="axrat"):
        O.evaluate(O.Case(10, 10, [("sersic", dict(axrat=0.0))]))
    with pytest.raises(O.OracleError, match="No psf provided"):
        O.evaluate(O.Case(10, 10, [("sersic", dict(convolve=True))]))
    with pytest.raises(O.OracleError, match="dimensions are 0"):
        O.evaluate(O.Case(0, 10, [("sersic", dict())]))
