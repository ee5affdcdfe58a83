"""Parameters written on the device are validated as the reference's
validate() does on every evaluate (src/radial.cpp:204-214 and each kind's
validate, e.g. src/sersic.cpp:207-218) (GPU).

A fitting loop writes parameters with pf_batch_set_params_dev or inside
pf_step_graph, where the host never sees them. The setup kernel checks every
profile with the reference's rules: pf_batch_check then fails with
PF_ERR_INVALID_PARAMETER and the reference's message (naming the first bad
profile), the bad profile draws nothing and gets no gradient, every other
model's image is the one a valid pass gives, and the next valid pass checks
clean again.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# (kind, parameter, slot, bad value, the reference's message)
CASES = [("sersic", "axrat", 4, 0.0, "axrat <= 0, must have axrat > 0"),
         ("sersic", "axrat", 4, 1.5, "axrat > 1, must have axrat <= 1"),
         ("sersic", "box", 5, -2.5, "box <= -2, must have box > -2"),
         ("sersic", "re", 6, -1.0, "re <= 0, must have re > 0"),
         ("sersic", "nser", 7, 0.0, "nser <= 0, must have nser > 0"),
         ("coresersic", "b", 10, 2.5, "b > 1.999, must have b < 1.999"),
         ("moffat", "con", 7, -0.5, "con < 0, must have con >= 0"),
         ("ferrer", "b", 8, 2.5, "b > 2, must have b <= 2"),
         ("king", "rt", 7, 0.0, "rt <= 0, must have rt > 0"),
         ("brokenexp", "h2", 7, -3.0, "h2 <= 0, must have h2 > 0")]


def _specs(kind):
    import workloads as W
    rng = np.random.default_rng(3)
    psf = W.moffat_psf(9, 2.5, 2.5)
    out = []
    for i in range(3):
        prof = [W._radial("sersic", rng, 48, 48, nser=2.0), W._radial(kind, rng, 48, 48, nser=1.5),
                ("sky", dict(bg=0.1))]
        out.append(dict(width=48, height=48, psf=psf, profiles=prof))
    return out


@pytest.mark.parametrize("use_double", [False, True])
@pytest.mark.parametrize("kind,name,slot,bad,msg", CASES, ids=["%s-%s-%g" % (c[0], c[1], c[3]) for c in CASES])
def test_invalid_parameters_on_device(kind, name, slot, bad, msg, use_double):
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    env = pg.get_cuda_environment(0, use_double=use_double)
    specs = _specs(kind)
    b = pg.Batch([W.to_model(s, env) for s in specs], env)
    dt = torch.float64 if use_double else torch.float32
    par = W.param_matrix(specs)
    pd = torch.tensor(par.ravel(), dtype=torch.float64, device="cuda")
    img = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
    b.set_params_dev(pd)
    b.forward(img)
    b.check()
    good = img.cpu().numpy().copy()
    # profile 4 is model 1's second profile (3 profiles per model)
    bad_par = par.copy()
    bad_par[4, slot] = bad
    b.set_params_dev(torch.tensor(bad_par.ravel(), dtype=torch.float64, device="cuda"))
    img.zero_()
    b.forward(img)
    with pytest.raises(pg.InvalidParameter) as e:
        b.check()
    assert str(e.value) == msg + " (profile 4 of the batch)"
    got = img.cpu().numpy()
    for i in (0, 2):  # the other models are untouched by the bad profile
        a, z = b.offsets[i], b.offsets[i + 1]
        np.testing.assert_array_equal(got[a:z], good[a:z])
    # model 1 without its bad profile: the sersic and the sky alone
    only = dict(specs[1], profiles=[specs[1]["profiles"][0], specs[1]["profiles"][2]])
    b1 = pg.Batch([W.to_model(only, env)], env)
    ref = torch.zeros(b1.total_pixels, dtype=dt, device="cuda")
    b1.forward(ref)
    b1.check()
    a, z = b.offsets[1], b.offsets[2]
    np.testing.assert_allclose(got[a:z], ref.cpu().numpy(), rtol=1e-6 if not use_double else 1e-12, atol=0)
    # valid again: no error left over
    b.set_params_dev(pd)
    b.forward(img)
    b.check()
    np.testing.assert_array_equal(img.cpu().numpy(), good)


def test_invalid_parameters_in_step_graph():
    """The same through pf_step_graph (parameters, forward, chi^2 and
    gradients as one graph launch): the error is reported, the bad profile's
    gradient is zero, and a later valid replay checks clean."""
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    env = pg.get_cuda_environment(0, use_double=False)
    specs = _specs("sersic")
    b = pg.Batch([W.to_model(s, env) for s in specs], env)
    b.enable_adjoint()
    par = W.param_matrix(specs)
    img = torch.zeros(b.total_pixels, dtype=torch.float32, device="cuda")
    b.forward(img)
    b.check()
    data = img.clone() * 1.01
    sigma = torch.full_like(img, 0.01 * float(img.max()))
    chi2 = torch.zeros(len(specs), dtype=torch.float64, device="cuda")
    grad = torch.zeros(b.n_profiles * 12, dtype=torch.float64, device="cuda")
    stream = torch.cuda.Stream()
    pgood = torch.tensor(par.ravel(), dtype=torch.float64, device="cuda")
    bad_par = par.copy()
    bad_par[4, 4] = 0.0  # axrat
    pbad = torch.tensor(bad_par.ravel(), dtype=torch.float64, device="cuda")
    pstep = pgood.clone()
    b.step_graph(pstep, img, data, sigma, chi2, grad, stream=stream)
    b.check(stream=stream)
    pstep.copy_(pbad)
    torch.cuda.synchronize()
    b.step_graph(pstep, img, data, sigma, chi2, grad, stream=stream)
    with pytest.raises(pg.InvalidParameter, match=r"^axrat <= 0, must have axrat > 0 \(profile 4 of the batch\)$"):
        b.check(stream=stream)
    g = grad.cpu().numpy().reshape(-1, 12)
    assert np.all(g[4] == 0)
    assert np.all(np.isfinite(g)) and np.all(np.isfinite(chi2.cpu().numpy()))
    pstep.copy_(pgood)
    torch.cuda.synchronize()
    b.step_graph(pstep, img, data, sigma, chi2, grad, stream=stream)
    b.check(stream=stream)


def test_environment_released_after_its_batches():
    """An environment closed while a batch still uses it (as garbage
    collection may order it) stays alive until that batch is destroyed: the
    batch still renders, and nothing is left behind for later calls."""
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    specs = _specs("sersic")
    env = pg.get_cuda_environment(0, use_double=False)
    b = pg.Batch([W.to_model(s, env) for s in specs], env)
    img = torch.zeros(b.total_pixels, dtype=torch.float32, device="cuda")
    b.forward(img)
    b.check()
    first = img.cpu().numpy().copy()
    env.close()
    img.zero_()
    b.forward(img)
    b.check()
    np.testing.assert_array_equal(img.cpu().numpy(), first)
    b.close()
    env2 = pg.get_cuda_environment(0, use_double=False)
    b2 = pg.Batch([W.to_model(s, env2) for s in specs], env2)
    b2.forward(img)
    b2.check()
    np.testing.assert_array_equal(img.cpu().numpy(), first)
