"""The autotuner's decision cache (GPU).

Single-precision batches time their choices: for PF_CONV_AUTO batches of at
least 2^22 output pixels, the convolution method per model and the block
shapes; for every batch, whether the subsampling trees split off to other
warps. An environment keeps those decisions by batch layout, as FFTW keeps
plans, and with PF_AUTOTUNE_CACHE naming a file it reads them from it and
appends new ones to it, as FFTW's wisdom outlives the process
(src/library.cpp:69-165 in the reference). A layout seen before is created
with the same decisions and no timing.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(env, n_models=64, side=256):
    import libprofit_gb300 as pg
    import workloads as W
    specs = [dict(s, width=side, height=side) for s in W.cfg4(n_models)]
    b = pg.Batch([W.to_model(s, env) for s in specs], env)
    b.enable_adjoint()
    return b


def _render(b):
    import torch
    img = torch.zeros(b.total_pixels, dtype=torch.float32, device="cuda")
    b.forward(img)
    b.check()
    return img.cpu().numpy()


@pytest.fixture(scope="module")
def built():
    import __graft_entry__
    __graft_entry__.build_cuda()


def test_same_layout_reused_in_environment(built):
    import libprofit_gb300 as pg
    env = pg.CUDAEnv(0, use_double=False)
    a = _batch(env)  # 64 models of 256 x 256: 2^22 output pixels, the full autotuner
    first = env.autotune_counts()
    assert first["timed"] >= 2 and first["reused"] == 0  # forward plan and split, adjoint shape
    b = _batch(env)
    second = env.autotune_counts()
    assert second["timed"] == first["timed"]
    assert second["reused"] >= 2
    assert a.conv_info() == b.conv_info()
    assert np.array_equal(_render(a), _render(b))
    # another layout (other image size) is timed anew
    _batch(env, n_models=64, side=264)
    assert env.autotune_counts()["timed"] > second["timed"]


def test_small_batch_split_decision_reused(built):
    import libprofit_gb300 as pg
    env = pg.CUDAEnv(0, use_double=False)
    _batch(env, n_models=2, side=128)
    first = env.autotune_counts()
    assert first["timed"] == 1 and first["reused"] == 0  # the split alone (no adjoint timing below 2^22)
    _batch(env, n_models=2, side=128)
    assert env.autotune_counts() == {"timed": 1, "reused": 1}


def test_cache_file_carries_decisions(built, tmp_path, monkeypatch):
    import libprofit_gb300 as pg
    path = tmp_path / "tune.txt"
    monkeypatch.setenv("PF_AUTOTUNE_CACHE", str(path))
    env_a = pg.CUDAEnv(0, use_double=False)
    a = _batch(env_a)
    lines = path.read_text().splitlines()
    assert lines and all(ln.startswith("pfcuda-tune 1 ") for ln in lines)
    # a new environment (as a new process would) reads the file: nothing timed
    env_b = pg.CUDAEnv(0, use_double=False)
    b = _batch(env_b)
    assert env_b.autotune_counts()["timed"] == 0
    assert env_b.autotune_counts()["reused"] >= 2
    assert a.conv_info() == b.conv_info()
    assert np.array_equal(_render(a), _render(b))
    # a file with a damaged line still loads its good lines
    path.write_text("pfcuda-tune 1 not-a-key\n" + "\n".join(lines) + "\n")
    env_c = pg.CUDAEnv(0, use_double=False)
    _batch(env_c)
    assert env_c.autotune_counts()["timed"] == 0
