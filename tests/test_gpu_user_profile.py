"""A user-defined radial profile compiled into the library (GPU).

libprofit takes new profiles as RadialProfile subclasses compiled into the
library (docs/new_profile.rst); this library takes them as a file of device
functions compiled in by `build.py --user-profile` (csrc/user_profile.cuh).
The example libprofit_gb300/user_profiles/example_moffat.cuh restates the
Moffat profile (src/moffat.cpp) as "usermoffat". A library built with it,
loaded in a separate process (PF_CUDA_LIBRARY), must render "usermoffat"
bit for bit as the built-in "moffat" -- itself equal to the compiled
reference to 1e-10 on the golden cases -- with the same subsampling counts;
validate its parameters with the plugin's messages on the host and on the
device; and refuse it in single precision and in the adjoint.
"""
import os
import subprocess
import sys

import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r'''
import numpy as np, torch
import libprofit_gb300 as pg
import workloads as W
from oracle import oracle as O
O.build(with_ref=False)
psf = W.moffat_psf(11, 2.5, 2.5)
env = pg.get_cuda_environment(0, use_double=True, profile=True)
for params in (dict(xcen=30.3, ycen=28.6, mag=14.0, fwhm=5.0, con=2.3, ang=40.0, axrat=0.6, box=0.0),
               dict(xcen=20.2, ycen=33.9, mag=16.0, fwhm=3.0, con=4.0, ang=10.0, axrat=0.9, box=0.3)):
    imgs, stats = {}, {}
    for kind in ("moffat", "usermoffat"):
        m = pg.Model(60, 60)
        m.set_cuda_env(env)
        m.set_psf(psf)
        p = m.add_profile(kind)
        for k, v in params.items():
            p.parameter(k, v)
        p.parameter("convolve", True)
        imgs[kind] = m.evaluate()
        stats[kind] = m.get_stats()[kind]
    assert np.array_equal(imgs["moffat"], imgs["usermoffat"]), "images differ"
    assert stats["moffat"]["integrations"] == stats["usermoffat"]["integrations"], "trees differ"
    assert stats["moffat"]["evaluations"] == stats["usermoffat"]["evaluations"]
    ref, _, _ = O.evaluate(O.Case(60, 60, [("moffat", dict(params, convolve=True))], psf=psf))
    got = imgs["usermoffat"]
    assert np.all(got[ref == 0] == 0)
    nz = ref != 0
    rel = np.max(np.abs(got[nz] - ref[nz]) / np.abs(ref[nz]))
    assert rel <= 1e-10, rel
# host validation with the plugin's message
m = pg.Model(20, 20)
m.set_cuda_env(env)
p = m.add_profile("usermoffat")
p.parameter("con", -1.0)
try:
    m.evaluate()
    raise SystemExit("con < 0 accepted")
except pg.InvalidParameter as e:
    assert str(e) == "con < 0, must have con >= 0", str(e)
# device validation (parameters written on the device)
spec = dict(width=20, height=20, profiles=[("usermoffat", dict(xcen=10.0, ycen=10.0, fwhm=3.0, con=2.0))])
b = pg.Batch([W.to_model(spec, env)], env)
par = torch.tensor([10.0, 10.0, 15.0, 0.0, 1.0, 0.0, -3.0, 2.0, 0, 0, 0, 0], dtype=torch.float64, device="cuda")
img = torch.zeros(b.total_pixels, dtype=torch.float64, device="cuda")
b.set_params_dev(par)
b.forward(img)
try:
    b.check()
    raise SystemExit("fwhm < 0 accepted on the device")
except pg.InvalidParameter as e:
    assert str(e) == "fwhm <= 0, must have fwhm > 0 (profile 0 of the batch)", str(e)
# single precision and the adjoint refuse it
env32 = pg.get_cuda_environment(0, use_double=False)
try:
    pg.Batch([W.to_model(spec, env32)], env32)
    raise SystemExit("single precision accepted")
except pg.Unsupported as e:
    assert "double precision only" in str(e)
b = pg.Batch([W.to_model(spec, env)], env)
try:
    b.enable_adjoint()
    raise SystemExit("adjoint accepted")
except pg.Unsupported:
    pass
print("user profile ok")
'''


def test_user_profile_library(tmp_path):
    import __graft_entry__
    __graft_entry__.build_cuda()
    from libprofit_gb300 import build
    plugin = os.path.join(ROOT, "libprofit_gb300", "user_profiles", "example_moffat.cuh")
    lib = build.build(user_profile=plugin, out_dir=str(tmp_path / "userlib"))
    env = dict(os.environ, PF_CUDA_LIBRARY=lib, PYTHONPATH=ROOT)
    r = subprocess.run([sys.executable, "-c", SCRIPT], env=env, capture_output=True, text=True, cwd=ROOT)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "user profile ok" in r.stdout
