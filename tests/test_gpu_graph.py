"""pf_step_graph (GPU): the fitting step captured once into a CUDA graph and
replayed gives, bit for bit, what the same calls give launched one by one;
replays follow the parameters written into the captured device buffer, and
parameters set on the host between launches."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(use_double):
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W
    env = pg.get_cuda_environment(0, use_double=use_double)
    specs = W.cfg4(6)
    for s in specs:
        s["width"] = s["height"] = 96
        for _, p in s["profiles"]:
            p["xcen"] *= 96 / 256
            p["ycen"] *= 96 / 256
    b = pg.Batch([W.to_model(s, env) for s in specs], env)
    b.enable_adjoint()
    dt = torch.float64 if use_double else torch.float32
    par = W.param_matrix(specs)
    rng = np.random.default_rng(3)
    data = torch.tensor(rng.random(b.total_pixels), dtype=dt, device="cuda")
    sigma = torch.full_like(data, 0.5)
    return torch, b, dt, par, data, sigma


def _eager(torch, b, dt, params, data, sigma, stream):
    img = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
    chi2 = torch.zeros(len(b.models), dtype=torch.float64, device="cuda")
    grad = torch.zeros(b.n_profiles * 12, dtype=torch.float64, device="cuda")
    b.set_params_dev(params, stream=stream.cuda_stream)
    b.forward_backward(img, data, sigma, chi2, grad, stream=stream.cuda_stream)
    stream.synchronize()
    return img.clone(), chi2.clone(), grad.clone()


@pytest.mark.parametrize("use_double", [False, True])
def test_graph_replays_match_eager(use_double):
    torch, b, dt, par, data, sigma = _setup(use_double)
    stream = torch.cuda.Stream()
    params = torch.tensor(par.ravel(), dtype=torch.float64, device="cuda")
    img = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
    chi2 = torch.zeros(len(b.models), dtype=torch.float64, device="cuda")
    grad = torch.zeros(b.n_profiles * 12, dtype=torch.float64, device="cuda")
    for step in range(3):
        p2 = par.copy()
        p2[:, 0] += 0.1 * step       # xcen of every profile
        p2[:, 6] *= 1 + 0.02 * step  # re / bg
        with torch.cuda.stream(stream):
            params.copy_(torch.tensor(p2.ravel(), dtype=torch.float64))
        b.step_graph(params, img, data, sigma, chi2, grad, stream=stream.cuda_stream)
        stream.synchronize()
        ref = _eager(torch, b, dt, torch.tensor(p2.ravel(), dtype=torch.float64, device="cuda"), data, sigma, stream)
        assert torch.equal(img, ref[0])
        assert torch.equal(chi2, ref[1])
        assert torch.equal(grad, ref[2])
    b.check(stream=stream.cuda_stream)


def test_graph_without_params_uses_host_parameters():
    torch, b, dt, par, data, sigma = _setup(False)
    stream = torch.cuda.Stream()
    img = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
    chi2 = torch.zeros(len(b.models), dtype=torch.float64, device="cuda")
    grad = torch.zeros(b.n_profiles * 12, dtype=torch.float64, device="cuda")
    b.step_graph(None, img, data, sigma, chi2, grad, stream=stream.cuda_stream)
    p2 = par.copy()
    p2[:, 2] += 0.3  # mag
    b.set_params(p2)
    b.step_graph(None, img, data, sigma, chi2, grad, stream=stream.cuda_stream)
    stream.synchronize()
    ref = _eager(torch, b, dt, torch.tensor(p2.ravel(), dtype=torch.float64, device="cuda"), data, sigma, stream)
    assert torch.equal(img, ref[0])
    assert torch.equal(grad, ref[2])


def test_graph_refuses_default_stream():
    torch, b, dt, par, data, sigma = _setup(False)
    import libprofit_gb300 as pg
    img = torch.zeros(b.total_pixels, dtype=dt, device="cuda")
    grad = torch.zeros(b.n_profiles * 12, dtype=torch.float64, device="cuda")
    with pytest.raises(pg.InvalidParameter):
        b.step_graph(None, img, data, sigma, None, grad, stream=0)
