"""profit-cli for the CUDA backend (libprofit_gb300/cli/profit_cli.cpp): the
reference's command line (src/profit-cli.cpp: -p profile specs, -P PSF, -f
FITS output, -t text output, -i timing iterations, -s stats, -T convolver, -u
uncropped) on this library.

CPU: it builds with the library, prints its usage and version, and refuses
unknown options. GPU: the reference's single-sersic model with its 15 x 15
Moffat PSF (given as a FITS file) written to a FITS file equals the compiled
reference's image to 1e-10; -i reports its iterations; -s the statistics of
Model::get_stats; -T fft -u the FFT convolver's uncropped frame, as
Model.evaluate_with_offset gives it.
"""
import os
import subprocess

import numpy as np
import pytest


def _cli():
    import __graft_entry__
    __graft_entry__.build_cuda()
    from libprofit_gb300 import build
    return build.build_cli()


def test_cli_usage_and_version():
    exe = _cli()
    r = subprocess.run([exe, "-h"], capture_output=True, text=True)
    assert r.returncode == 0 and "Usage:" in r.stdout and "-p <spec>" in r.stdout
    r = subprocess.run([exe, "-V"], capture_output=True, text=True)
    assert r.returncode == 0 and "sm_103a" in r.stdout
    r = subprocess.run([exe, "-q"], capture_output=True, text=True)
    assert r.returncode == 1
    r = subprocess.run([exe], capture_output=True, text=True)  # no profile
    assert r.returncode == 1 and "Usage:" in r.stdout


SERSIC = "sersic:xcen=50.3:ycen=50.7:mag=15:re=8:nser=4:ang=30:axrat=0.6:box=0:convolve=1"


@pytest.mark.gpu
def test_cli_reference_model(tmp_path):
    import libprofit_gb300 as pg
    from tests.golden.load import load
    golden = load()["cfg1_sersic_brute"]
    exe = _cli()
    psf = str(tmp_path / "psf.fits")
    pg.to_fits(np.asarray(golden["psf"], dtype=np.float64), (0, 0), (1.0, 1.0), psf)
    out = str(tmp_path / "out.fits")
    r = subprocess.run([exe, "-w", "100", "-H", "100", "-p", SERSIC, "-P", psf, "-T", "brute", "-f", out, "-i", "3",
                        "-s"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "Ran 3 iterations in" in r.stdout
    img, scale = pg.from_fits(out)
    ref = golden["image"]
    assert img.shape == ref.shape
    assert np.max(np.abs(img - ref) / np.abs(ref)) <= 1e-10
    assert "Stats for profile sersic" in r.stdout
    calls = int(r.stdout.split("evaluate_at calls:")[1].split()[0])
    assert calls > 0


@pytest.mark.gpu
def test_cli_fft_uncropped(tmp_path):
    import libprofit_gb300 as pg
    import workloads as W
    exe = _cli()
    psf = W.moffat_psf(9, 2.5, 2.5)
    vals = ",".join("%.17g" % v for v in psf.ravel())
    r = subprocess.run([exe, "-w", "40", "-H", "40", "-p", "sersic:xcen=20.3:ycen=19.8:re=4:nser=2.2:convolve=1",
                        "-P", "9:9:" + vals, "-T", "fft", "-u", "-t"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    rows = [ln.split() for ln in r.stdout.splitlines() if ln and ln[0] in "0123456789-"]
    img = np.array([[float(v) for v in row] for row in rows])
    m = pg.Model(40, 40)
    m.set_psf(psf)
    m.set_convolver("fft")
    m.set_crop(False)
    p = m.add_profile("sersic")
    for k, v in dict(xcen=20.3, ycen=19.8, re=4.0, nser=2.2).items():
        p.parameter(k, v)
    p.parameter("convolve", True)
    want, _ = m.evaluate_with_offset()
    assert img.shape == want.shape
    np.testing.assert_allclose(img, want, rtol=1e-5, atol=1e-5 * np.abs(want).max())
