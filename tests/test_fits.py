"""FITS images in and out (host code of libpfcuda.so; no GPU needed).

pf_fits_write / pf_fits_read against the reference's to_fits / from_fits
(src/fits_utils.cpp:60-205), through the fixtures in tests/golden/fits/
written by the reference (tests/golden/make_fits_golden.py):
  * every file this library writes is byte-for-byte the reference's;
  * every reference file reads back to the reference's from_fits result bit
    for bit (signed zeros, subnormals, infinities included), with its pixel
    scale (CDELT written with six decimals, as the reference writes it);
  * ".fits" is appended unless the name ends in it;
  * missing, truncated and short files raise InvalidFile with the
    reference's messages.
Where the reference compiled here (oracle/_ref), each direction is also
checked live against it.
"""
import json
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
FITS_DIR = os.path.join(ROOT, "tests", "golden", "fits")


def _manifest():
    m = np.load(os.path.join(FITS_DIR, "manifest.npz"))
    meta = json.loads(str(m["meta"]))
    return m, meta


MANIFEST, META = _manifest()
NAMES = sorted(k for k in META if not k.startswith("_"))


@pytest.fixture(scope="module")
def pg():
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300
    return libprofit_gb300


def _ref_available():
    return os.path.exists(os.path.join(ROOT, "oracle", "_ref", "libprofit_ref.so"))


def _bits(a):
    return np.ascontiguousarray(a, dtype=np.float64).view(np.uint64)


@pytest.mark.parametrize("name", NAMES)
def test_write_matches_reference_bytes(pg, tmp_path, name):
    img = MANIFEST["image_" + name]
    meta = META[name]
    out = tmp_path / (name + ".fits")
    pg.to_fits(img, meta["offset"], meta["scale"], str(out))
    got = out.read_bytes()
    want = open(os.path.join(FITS_DIR, name + ".fits"), "rb").read()
    assert len(got) == meta["bytes"] == len(want)
    assert got == want


@pytest.mark.parametrize("name", NAMES)
def test_read_matches_reference(pg, name):
    img, scale = pg.from_fits(os.path.join(FITS_DIR, name + ".fits"))
    want = MANIFEST["read_" + name]
    assert img.shape == want.shape
    assert np.array_equal(_bits(img), _bits(want))
    assert list(scale) == META[name]["read_scale"]
    # the pixels are the written ones exactly; the scale as CDELT's 6 decimals
    assert np.array_equal(_bits(img), _bits(MANIFEST["image_" + name]))


def test_suffix_rule(pg, tmp_path, monkeypatch):
    """The rule looks at the name as given (a path of more than five
    characters ending in ".fits" keeps it)."""
    monkeypatch.chdir(tmp_path)
    img = np.ones((2, 3))
    for given, written in [("a", "a.fits"), ("b.fits", "b.fits"), ("c.fit", "c.fit.fits"),
                           (".fits", ".fits.fits"), ("d.FITS", "d.FITS.fits")]:
        pg.to_fits(img, (0, 0), (1, 1), given)
        assert (tmp_path / written).exists(), given
    with pytest.raises(pg.InvalidParameter):
        pg.to_fits(img, (0.5, 0), (1, 1), "e")
    with pytest.raises(pg.InvalidParameter):
        pg.to_fits(img, (-1, 0), (1, 1), "e")


def test_failures(pg, tmp_path, monkeypatch):
    msgs = META["_failures"]
    monkeypatch.chdir(tmp_path)
    with pytest.raises(pg.InvalidFile) as e:
        pg.from_fits("missing.fits")
    assert str(e.value) == msgs["missing.fits"]
    with open("header_cut.fits", "wb") as f:
        f.write(b"SIMPLE  =                    T".ljust(80) + b"NAXIS1  = 4".ljust(40))
    with pytest.raises(pg.InvalidFile) as e:
        pg.from_fits("header_cut.fits")
    assert str(e.value) == msgs["header_cut.fits"]
    pg.to_fits(np.ones((4, 4)), (0, 0), (1, 1), "short_data.fits")
    data = open("short_data.fits", "rb").read()
    with open("short_data.fits", "wb") as f:
        f.write(data[:2880 + 100])
    with pytest.raises(pg.InvalidFile) as e:
        pg.from_fits("short_data.fits")
    assert str(e.value) == msgs["short_data.fits"]
    with pytest.raises(pg.InvalidFile, match="for writing"):
        pg.to_fits(np.ones((1, 1)), (0, 0), (1, 1), str(tmp_path / "no_such_dir" / "x"))


def test_round_trip_large(pg, tmp_path):
    """A 1000 x 700 image (several 64 KiB write/read chunks) round-trips."""
    rng = np.random.Generator(np.random.PCG64(7))
    img = rng.standard_normal((700, 1000))
    pg.to_fits(img, (1, 2), (0.25, 0.5), str(tmp_path / "big"))
    back, scale = pg.from_fits(str(tmp_path / "big.fits"))
    assert np.array_equal(back, img) and scale == (0.25, 0.5)
    assert (tmp_path / "big.fits").stat().st_size % 2880 == 0


@pytest.mark.skipif(not _ref_available(), reason="the reference is compiled only where its sources are")
def test_live_against_reference(pg, oracle_lib, tmp_path):
    O = oracle_lib
    rng = np.random.Generator(np.random.PCG64(11))
    for w, h in [(1, 1), (5, 3), (40, 36), (123, 77)]:
        img = rng.standard_normal((h, w)) * 1e3
        offset = (int(rng.integers(0, 50)), int(rng.integers(0, 50)))
        scale = (rng.uniform(0.1, 3), rng.uniform(0.1, 3))
        O.ref_to_fits(img, offset, scale, str(tmp_path / "ref"))
        pg.to_fits(img, offset, scale, str(tmp_path / "ours"))
        assert (tmp_path / "ref.fits").read_bytes() == (tmp_path / "ours.fits").read_bytes()
        a, sa = pg.from_fits(str(tmp_path / "ref.fits"))
        b, sb = O.ref_from_fits(str(tmp_path / "ours.fits"))
        assert np.array_equal(a, b) and sa == sb
