"""Parity cases shared by the golden-fixture generator and the tests.

Each case is a plain dict: model settings plus a list of (profile kind,
parameters) in the order Model::add_profile would receive them. The parameter
names are the reference's own (Profile::parameter, src/profile.cpp:69-163;
defaults from src/radial.cpp:724-752 and each profile's constructor).
Cases follow the reference's own test fixtures where it has them:
tests/test_radial.h:65-89 (all radial profiles, default and boxy, centred at
50,50 on 100x100), tests/test_sersic.h:36-51 (nser in {0.5..16}, box 0 and
0.1 on 50x50), tests/test_psf.h:38-50 (2x2 uniform PSF known answer),
tests/test_sky.h:37-61 (sky known answer), tests/test_model.h:204-303
(profile addition, finesampling), plus the 100x100 single-Sersic model with a
15x15 Moffat PSF.
"""
import numpy as np

RADIAL = ["sersic", "coresersic", "moffat", "ferrer", "king", "brokenexp"]


def moffat_psf_case(size, fwhm, con):
    """The model that renders a centred size x size Moffat PSF."""
    return dict(width=size, height=size,
                profiles=[("moffat", dict(xcen=size / 2.0, ycen=size / 2.0, fwhm=fwhm, con=con, mag=0.0))])


def golden_cases():
    """Returns {name: case dict}. PSFs are given as the name of another case
    (rendered first) or an explicit array."""
    c = {}
    c["psf15_moffat"] = moffat_psf_case(15, 3.0, 2.5)
    c["cfg1_sersic_nopsf"] = dict(width=100, height=100, profiles=[
        ("sersic", dict(xcen=50.3, ycen=50.7, mag=15, re=8, nser=4, ang=30, axrat=0.6, box=0))])
    c["cfg1_sersic_brute"] = dict(width=100, height=100, psf="psf15_moffat", profiles=[
        ("sersic", dict(xcen=50.3, ycen=50.7, mag=15, re=8, nser=4, ang=30, axrat=0.6, box=0,
                        convolve=True))])
    for k in RADIAL:
        c["%s_default" % k] = dict(width=100, height=100, profiles=[(k, dict(xcen=50.0, ycen=50.0))])
        c["%s_boxy" % k] = dict(width=100, height=100, profiles=[(k, dict(xcen=50.0, ycen=50.0, box=0.1))])
        c["%s_rotated" % k] = dict(width=64, height=48, profiles=[
            (k, dict(xcen=20.3, ycen=27.9, ang=71.0, axrat=0.45, box=-0.3))])
    extra = {
        "sersic": dict(re=6.0, nser=2.7),
        "coresersic": dict(re=7.0, rb=1.5, nser=3.0, a=2.0, b=0.5),
        "moffat": dict(fwhm=4.0, con=3.3),
        "ferrer": dict(rout=12.0, a=1.5, b=0.7),
        "king": dict(rc=2.5, rt=14.0, a=2.2),
        "brokenexp": dict(h1=3.0, h2=1.5, rb=6.0, a=1.3),
    }
    for k, ex in extra.items():
        p = dict(xcen=30.6, ycen=25.2, ang=133.0, axrat=0.7, mag=17.5)
        p.update(ex)
        c["%s_shaped" % k] = dict(width=60, height=52, profiles=[(k, p)])
    for n in [0.5, 1.0, 1.5, 2.0, 3.0, 4.0, 8.0, 16.0]:
        for box in (0.0, 0.1):
            c["sersic_n%s_box%s" % (n, box)] = dict(width=50, height=50, profiles=[
                ("sersic", dict(xcen=25.0, ycen=25.0, nser=n, box=box))])
    c["sersic_rough"] = dict(width=40, height=40, profiles=[
        ("sersic", dict(xcen=20.2, ycen=19.6, re=4.0, nser=2.0, rough=True))])
    c["sersic_noadjust"] = dict(width=40, height=40, profiles=[
        ("sersic", dict(xcen=20.2, ycen=19.6, re=4.0, nser=2.5, adjust=False, resolution=5,
                        max_recursions=3, acc=0.05, rscale_switch=1.5, rscale_max=6.0))])
    c["sersic_rescale_flux"] = dict(width=50, height=50, profiles=[
        ("sersic", dict(xcen=24.1, ycen=26.3, re=5.0, nser=3.0, rescale_flux=True))])
    c["sersic_scale_magzero"] = dict(width=50, height=40, scale=(0.5, 0.7), magzero=25.0, profiles=[
        ("sersic", dict(xcen=12.3, ycen=14.1, re=3.0, nser=1.7, ang=15.0, axrat=0.8, mag=20.0))])
    c["addition_three_sersics"] = dict(width=100, height=100, profiles=[
        ("sersic", dict(xcen=50.0, ycen=50.0, re=10.0)),
        ("sersic", dict(xcen=30.0, ycen=10.0, re=16.0)),
        ("sersic", dict(xcen=23.0, ycen=89.0, re=1.2))])
    c["finesampled"] = dict(width=40, height=30, finesampling=2, profiles=[
        ("sersic", dict(xcen=20.0, ycen=15.0, re=5.0, nser=2.0))])
    c["finesampled_downsampled"] = dict(width=40, height=30, finesampling=3, return_finesampled=False,
                                        profiles=[("moffat", dict(xcen=21.0, ycen=13.5, fwhm=3.0, con=2.2))])
    c["psf_known_answer"] = dict(width=10, height=10, psf=np.ones((2, 2)).tolist(), profiles=[
        ("psf", dict(xcen=2.0, ycen=2.0, mag=0.0))])
    c["sky_known_answer"] = dict(width=2, height=2, profiles=[("sky", dict(bg=1.0))])
    c["mixed_conv_sky_psf"] = dict(width=80, height=70, psf="psf15_moffat", profiles=[
        ("sersic", dict(xcen=40.3, ycen=33.7, mag=16, re=5, nser=3, ang=40, axrat=0.5, convolve=True)),
        ("moffat", dict(xcen=20.6, ycen=50.1, mag=18, fwhm=2.5, con=3.0, convolve=True)),
        ("sky", dict(bg=1e-3)),
        ("psf", dict(xcen=60.2, ycen=20.7, mag=19))])
    c["conv_brute_old"] = dict(width=50, height=50, psf="psf15_moffat", convolver="brute_old", profiles=[
        ("king", dict(xcen=25.5, ycen=24.5, rc=2.0, rt=12.0, convolve=True))])
    c["conv_even_psf"] = dict(width=45, height=50, psf=[[0.0, 1.0], [2.0, 3.0]], profiles=[
        ("sersic", dict(xcen=30.0, ycen=10.0, re=16.0, convolve=True))])
    # calculation masks (Model::set_mask, adjusted by Model::evaluate,
    # src/model.cpp:152-257): far from the edges (no PSF padding needed), on
    # an edge (padding needed), without convolution, finesampled and
    # SUM-downsampled, with sky and psf profiles, all zero, and random
    rng = np.random.default_rng(77)
    central = np.zeros((60, 60), np.uint8)
    central[15:45, 12:48] = 1
    c["mask_central_conv"] = dict(width=60, height=60, psf="psf15_moffat", mask=central.tolist(), profiles=[
        ("sersic", dict(xcen=30.3, ycen=29.6, mag=16, re=6, nser=3.5, ang=20, axrat=0.7, convolve=True))])
    edge = np.zeros((50, 60), np.uint8)
    edge[0:21, 30:60] = 1
    c["mask_edge_conv"] = dict(width=60, height=50, psf="psf15_moffat", mask=edge.tolist(), profiles=[
        ("sersic", dict(xcen=44.2, ycen=10.7, mag=16, re=5, nser=2.2, ang=60, axrat=0.5, convolve=True))])
    c["mask_nopsf"] = dict(width=50, height=50, mask=(rng.random((50, 50)) < 0.7).astype(np.uint8).tolist(),
                           profiles=[("sersic", dict(xcen=24.6, ycen=25.3, re=4.0, nser=2.5))])
    fsm = np.zeros((30, 40), np.uint8)
    fsm[8:24, 10:33] = 1
    c["mask_fs_downsampled"] = dict(width=40, height=30, finesampling=2, return_finesampled=False,
                                    psf="psf15_moffat", mask=fsm.tolist(), profiles=[
        ("moffat", dict(xcen=21.0, ycen=13.5, fwhm=3.0, con=2.2, convolve=True))])
    sky = np.ones((40, 50), np.uint8)
    sky[:, :9] = 0
    sky[31:, :] = 0
    c["mask_sky_psf_profile"] = dict(width=50, height=40, psf="psf15_moffat", mask=sky.tolist(), profiles=[
        ("sersic", dict(xcen=25.5, ycen=19.0, mag=17, re=4, nser=1.5, convolve=True)),
        ("sky", dict(bg=2e-3)),
        ("psf", dict(xcen=40.2, ycen=12.6, mag=18))])
    c["mask_all_zero"] = dict(width=30, height=30, psf="psf15_moffat", mask=np.zeros((30, 30), np.uint8).tolist(),
                              profiles=[("sersic", dict(xcen=15.0, ycen=15.0, re=4, convolve=True))])
    c["mask_random_conv"] = dict(width=64, height=56, psf="psf15_moffat",
                                 mask=(rng.random((56, 64)) < 0.5).astype(np.uint8).tolist(), profiles=[
        ("sersic", dict(xcen=30.1, ycen=25.9, mag=16, re=8, nser=4, ang=35, axrat=0.6, convolve=True)),
        ("sersic", dict(xcen=36.4, ycen=30.2, mag=15.5, re=14, nser=1, ang=110, axrat=0.4, box=0.1,
                        convolve=True)),
        ("sky", dict(bg=1e-3))])
    # masks used as given (Model::set_adjust_mask(false)): drawing dimensions,
    # with the PSF padding when the mask is larger than the model
    # (src/model.cpp:165-167, 277-283), without it otherwise
    padded = (rng.random((64, 74)) < 0.8).astype(np.uint8)
    padded[:, :6] = 0
    c["mask_given_padded"] = dict(width=60, height=50, psf="psf15_moffat", mask=padded.tolist(), adjust_mask=False,
                                  profiles=[
        ("sersic", dict(xcen=31.2, ycen=24.6, mag=15, re=6, nser=2.5, ang=40, axrat=0.6, box=0.1, convolve=True)),
        ("sky", dict(bg=0.01))])
    unpadded = np.ones((40, 50), np.uint8)
    unpadded[10:20, 5:45] = 0
    c["mask_given_unpadded"] = dict(width=50, height=40, psf="psf15_moffat", mask=unpadded.tolist(),
                                    adjust_mask=False, profiles=[
        ("sersic", dict(xcen=24.2, ycen=20.9, mag=15, re=7, nser=1.8, ang=100, axrat=0.8, convolve=True))])
    fine = (rng.random((50, 60)) < 0.6).astype(np.uint8)
    c["mask_given_finesampled"] = dict(width=30, height=25, finesampling=2, mask=fine.tolist(), adjust_mask=False,
                                       profiles=[("king", dict(xcen=14.8, ycen=12.2, rc=2.0, rt=9.0))])
    return c


def resolve_psf(case, rendered):
    psf = case.get("psf")
    if psf is None:
        return None
    if isinstance(psf, str):
        return rendered[psf]
    return np.asarray(psf, dtype=np.float64)
