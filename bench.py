"""Benchmark: batched model + VJP evaluations per second on one GB300.

Workload (default): 1024 models of 256x256 pixels, each a sersic bulge
(nser U[2,6]) plus a sersic disk (nser U[0.7,1.3]) convolved with a 25x25
Moffat PSF; data = the model at parameters perturbed by N(0, 5 %) plus
Gaussian noise (sigma = 1 % of each model's peak); one step = upload the
parameter vector, render every model (FP32 values, FP64 geometry and
decisions), chi^2 per model and d chi^2 / d (all 16 parameters of every
model) in FP64. Inputs are synthetic and seeded (workloads.py).

Other workloads (--workload, one JSON line each, same keys):
  cfg2  one 1000x1000 model (bulge + disk + sky, 51x51 PSF by FFT): FP32 and
        FP64 forward, models/s, with the FP32 result's errors against FP64;
  cfg3  4096 uneven models (1-3 of the six radial kinds, own PSFs, method by
        the autotuner): FP32 forward of the whole batch, models/s;
  cfg5  the 4096x4096 field with 10,000 profiles and a sky, 101x101 PSF by an
        4608x4608 FFT: FP32 forward + chi^2 + gradients of all 10,001
        profiles, fields/s.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                       [--workload cfg4|cfg2|cfg3|cfg5]
Under torchrun each rank renders its own copy of the workload (weak scaling,
no collective on the data path); rank 0 prints one JSON line.
--impl reference times the CPU oracle port of the reference's
Model::evaluate (OpenMP over all host cores) on a bounded sample of the same
workload, gradients by central differences (2 x 16 + 1 evaluations per model).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "batched model+VJP evals/s (FP32, ≤1e-5 rel flux err) vs plain FP64 GPU; Mpix/s"
N_PAR_MODEL = 16


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--models", type=int, default=None,
                    help="models in the batch (default: 1024 for cfg4, 4096 for cfg3)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-dropin", action="store_true", help="skip the one-model-per-call drop-in timings")
    ap.add_argument("--convolver", default="auto", choices=["auto", "brute", "fft"],
                    help="convolution method of the FP32 batch (auto: the library's choice)")
    ap.add_argument("--no-graph", action="store_true",
                    help="launch the step's kernels one by one instead of replaying its CUDA graph")
    ap.add_argument("--workload", default="cfg4", choices=["cfg4", "cfg2", "cfg3", "cfg5", "dropin"],
                    help="cfg4 (default): the batched model + VJP step; the others: see the module docstring")
    return ap.parse_args()


def dist_init(args, backend=None):
    """One process per GPU (torchrun's RANK / LOCAL_RANK / WORLD_SIZE): the
    ranks render independent replicas of the workload; the process group only
    carries the timing barrier and the max over ranks (NCCL on GPUs, gloo
    without). The reference arm, CPU only, starts none: rank 0 alone works."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1 and getattr(args, "impl", "ours") != "reference":
        import torch
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        if backend is None:
            backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(world, value):
    if world == 1:
        return value
    import torch
    import torch.distributed as dist
    on_gpu = dist.get_backend() == "nccl"
    t = torch.tensor([value], dtype=torch.float64, device="cuda" if on_gpu else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.FIELDS,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.thread.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def fft_length(n):
    """The single-precision FFT's transform length for n points: the smallest
    of 2^a (64 .. 8192) and 3, 5, 9 x 2^a (2^a >= 32) that is >= n."""
    lengths = sorted({1 << a for a in range(6, 14)} |
                     {f << a for f, top in ((3, 6144), (5, 5120), (9, 4608)) for a in range(5, 14) if f << a <= top})
    return next(x for x in lengths if x >= n)


def hbm_peak():
    """The measured copy bandwidth (MEASURED_PEAKS.json next to this file), or
    the 6.8 TB/s fallback."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return {"gbs": float(json.load(f)["hbm_gbs"]), "note": "of measured"}
    except (OSError, KeyError, ValueError):
        return {"gbs": 6800.0, "note": "of fallback"}


def make_problem(models, seed_offset, env64, torch):
    """Workload specs, the batch parameter matrix and the data (rendered by
    the FP64 path at perturbed parameters, plus noise)."""
    import libprofit_gb300 as pg
    import workloads as W
    specs = W.cfg4(models)
    par = W.param_matrix(specs)
    rng = np.random.Generator(np.random.PCG64(4000 + seed_offset))
    pert = par.copy()
    pert[:, :8] *= 1 + 0.05 * rng.standard_normal((pert.shape[0], 8))
    pert[:, 4] = np.clip(pert[:, 4], 0.05, 1.0)  # axrat stays valid
    pert[:, 7] = np.clip(pert[:, 7], 0.3, 10.0)
    b64 = pg.Batch([W.to_model(s, env64) for s in specs], env64)
    b64.set_params(pert)
    img64 = torch.zeros(b64.total_pixels, dtype=torch.float64, device="cuda")
    b64.forward(img64)
    b64.check()
    data = img64.cpu().numpy()
    sigma = np.empty_like(data)
    for i in range(len(specs)):
        a, z = b64.offsets[i], b64.offsets[i + 1]
        s = 0.01 * data[a:z].max()
        sigma[a:z] = s
        data[a:z] += rng.normal(0, s, z - a)
    b64.close()
    return specs, par, data, sigma


def cpu_baseline_sample(specs, par, budget_s=8.0):
    """Oracle port (C restatement of the reference CPU path, OpenMP on every
    host core): forward + central-difference gradient (2*16+1 evaluations) per
    model on a bounded sample of the workload's models. Returns models/s."""
    from oracle import oracle as O
    import workloads as W
    O.build(with_ref=False)
    threads = os.cpu_count() or 1
    t0 = time.time()
    done = 0
    rows = 0
    for s in specs:
        n = len(s["profiles"])
        case = W.to_oracle_case(s)
        O.evaluate(case, threads=threads)
        for j in range(n):
            kind, params = s["profiles"][j]
            for k in ("xcen", "ycen", "mag", "ang", "axrat", "box", "re", "nser"):
                for sgn in (1, -1):
                    p2 = dict(params)
                    p2[k] = p2[k] + sgn * 1e-6 * max(abs(p2[k]), 1e-3)
                    profs = list(s["profiles"])
                    profs[j] = (kind, p2)
                    O.evaluate(O.Case(s["width"], s["height"], profs, psf=s.get("psf")), threads=threads)
        done += 1
        rows += n
        if time.time() - t0 > budget_s:
            break
    dt = time.time() - t0
    return done / dt, threads, done, dt


def run_reference(args, world, rank):
    """--impl reference: the CPU oracle port on the host cores, rank 0 only."""
    if rank != 0:
        return
    import workloads as W
    specs = W.cfg4(args.models or 1024)
    par = W.param_matrix(specs)
    # K timed steps, each a bounded sample (rendering consecutive models from a
    # different start until its time budget runs out), the whole run about a
    # minute; W untimed warm-up steps of one model
    budget = min(5.0, max(0.5, 60.0 / max(1, args.steps)))
    vals = []
    for _ in range(args.warmup):
        cpu_baseline_sample(specs[:1], par, budget_s=0.05)
    t_all = time.time()
    for step in range(args.steps):
        start = (step * 37) % len(specs)
        v, threads, done, dt = cpu_baseline_sample(specs[start:] + specs[:start], par, budget_s=budget)
        vals.append(v)
    value = statistics.median(vals)
    line = {"metric": METRIC, "value": value, "unit": "models/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": "1024 models 256x256, sersic bulge+disk, 25x25 Moffat PSF, model+VJP",
                       "models": len(specs)},
            "cpu_baseline": {"value": value, "unit": "models/s", "cores": threads, "kind": "port",
                             "sample": "per step, consecutive models rendered + 33-point central-difference "
                                       "gradient until %.1f s have passed; median over the steps" % budget},
            "e2e": {"value": value, "unit": "models/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "wall_s": time.time() - t_all}
    print(json.dumps(line), flush=True)


# FP32-pipe work per evaluate_at of the sersic profile, counted from
# profiles_f32.cuh / eval_f32.cu (FMA = 2 flops, other FP32 ops 1, each MUFU
# op weighted 8, its issue cost against the FMA pipe: 128 vs 16 per SM-clock).
FLOP_EVAL = 2 * 7 + 5 + 3 * 8        # coordinates + base + rf + exp: 43
FLOP_GRAD = FLOP_EVAL + 40 + 4 * 8   # + the derivative chain (sersic_grad): 115
def dropin_rates(env64, env32, budget_s=2.0, cpu=True):
    """The drop-in path: Model.evaluate (pf_model_evaluate, host buffers in
    and out) on one model per call, the first sersic's xcen and nser changed
    between calls as a fitter changes parameters (so that the setup's solves
    are redone every call), for the one-model workloads (cfg1: 100x100,
    15x15 PSF, direct convolution; cfg2: 1000x1000 bulge + disk + sky, 51x51
    PSF by FFT), in the plain FP64 and the FP32 environments; and the CPU
    oracle port (all host threads) on the same models. Calls per second, each
    leg timed for about budget_s after three warm-up calls."""
    import workloads as W
    if cpu:
        from oracle import oracle as O
        O.build(with_ref=False)
    threads = os.cpu_count() or 1
    out = {"calls": "Model.evaluate through pf_model_evaluate with host buffers, one model per call",
           "cpu_threads": threads}
    for name, spec in (("cfg1", W.cfg1()[0]), ("cfg2", W.cfg2()[0])):
        row = {}
        for label, env in (("fp64", env64), ("fp32", env32)):
            m = W.to_model(spec, env)
            p = m.profiles[0]
            x0, n0 = spec["profiles"][0][1]["xcen"], spec["profiles"][0][1]["nser"]

            def call(k):
                p.parameter("xcen", x0 + 0.01 * (k % 7))
                p.parameter("nser", n0 * (1 + 1e-6 * (k % 5)))
                m.evaluate()
            k = 0
            for _ in range(3):
                call(k)
                k += 1
            n, t0 = 0, time.perf_counter()
            while time.perf_counter() - t0 < budget_s or n < 3:
                call(k)
                n += 1
                k += 1
            row[label + "_calls_per_s"] = n / (time.perf_counter() - t0)
        out[name] = row
        if not cpu:
            continue
        case = W.to_oracle_case(spec)
        O.evaluate(case, threads=threads)
        n, t0 = 0, time.perf_counter()
        while time.perf_counter() - t0 < budget_s or n < 1:
            O.evaluate(case, threads=threads)
            n += 1
        row["cpu_port_calls_per_s"] = n / (time.perf_counter() - t0)
        out[name] = row
    return out


# models whose images, chi^2 and gradients are checked against the plain FP64 path
ACC_MODELS = 32


def gradient_accuracy(specs, par, img64, data, sigma, g32, g64, env64):
    """The FP32 batch's gradients (n_profiles x 8) against the plain FP64
    path's on the same models and data: the largest relative error with no
    floor, the share of components within 1e-4 relative, and the check
    |g32 - g64| <= 1e-4 |g64| + 2e-6 sum_p |c_p dm_p/dpar| + 2e-6 sum_p
    2 |m_p dm_p/dpar| / sigma_p^2 (the scale of the sum each component is, and
    its sensitivity to the FP32 image's relative error; central differences
    of the FP64 path), over the components whose differences keep the
    subsampling tree."""
    import workloads as W
    scale_c, scale_m, same = W.gradient_scales(specs, par, img64, data, sigma, env64)
    err = np.abs(g32 - g64)
    rel = err / np.abs(g64)
    bound = 1e-4 * np.abs(g64) + 2e-6 * scale_c + 2e-6 * scale_m
    worst = np.unravel_index(np.argmax(rel), rel.shape)
    return {"models": len(specs), "components": int(rel.size),
            "max_rel_err": float(rel.max()),
            "median_rel_err": float(np.median(rel)),
            "frac_within_1e-4": float((rel <= 1e-4).mean()),
            "worst": {"g64": float(g64[worst]), "g32": float(g32[worst]),
                      "sum_abs_c_dm": float(scale_c[worst]), "sum_abs_2m_dm_over_sigma2": float(scale_m[worst])},
            "max_err_over_sum_abs_c_dm": float((err / scale_c)[same].max()),
            "max_err_over_sum_abs_2m_dm_over_sigma2": float((err / scale_m)[same].max()),
            "bound": "1e-4 |g64| + 2e-6 sum_p |c_p dm_p/dpar| + 2e-6 sum_p 2 |m_p dm_p/dpar| / sigma_p^2",
            "max_err_over_bound": float((err / bound)[same].max()),
            "components_checked": int(same.sum())}


# DRAM bytes per model of the adjoint direct convolution's launch (ncu, 256-model copy of the workload)
ADJ_CONV_TRAFFIC_PER_MODEL = (68.1e6 + 27.3e6) / 256


def run_ours(args, world, rank, local):
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W

    torch.cuda.set_device(local)
    env64 = pg.get_cuda_environment(local, use_double=True)
    env32 = pg.get_cuda_environment(local, use_double=False, profile=True)
    specs, par, data_np, sigma_np = make_problem(args.models or 1024, rank, env64, torch)
    n_models = len(specs)
    models32 = [W.to_model(s, env32) for s in specs]
    for m in models32:
        m.set_convolver(args.convolver)
    batch = pg.Batch(models32, env32)
    batch.enable_adjoint()
    n_prof = batch.n_profiles
    img = torch.zeros(batch.total_pixels, dtype=torch.float32, device="cuda")
    data = torch.tensor(data_np, dtype=torch.float32, device="cuda")
    sigma = torch.tensor(sigma_np, dtype=torch.float32, device="cuda")
    chi2 = torch.zeros(n_models, dtype=torch.float64, device="cuda")
    grad = torch.zeros(n_prof * 12, dtype=torch.float64, device="cuda")
    params = torch.tensor(par.ravel(), dtype=torch.float64, device="cuda")
    # consecutive steps alternate between the parameters and a copy moved by
    # ~1e-6 relative in every entry (nser included), as an optimiser's steps
    # are: nothing the setup caches across unchanged parameters carries over
    alt_np = par * (1 + 1e-6 * np.random.Generator(np.random.PCG64(6000 + rank)).standard_normal(par.shape))
    alt_np[:, 4] = np.minimum(alt_np[:, 4], 1.0)  # axrat stays <= 1
    p_alt = [params.clone(), torch.tensor(alt_np.ravel(), dtype=torch.float64, device="cuda")]
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    n_step = [0]

    def step():
        with torch.cuda.stream(stream):
            params.copy_(p_alt[n_step[0] & 1], non_blocking=True)
        n_step[0] += 1
        if args.no_graph:
            batch.set_params_dev(params, stream=sh)
            batch.forward_backward(img, data, sigma, chi2, grad, stream=sh)
        else:  # pf_step_graph: the same nine kernels, one graph launch
            batch.step_graph(params, img, data, sigma, chi2, grad, stream=sh)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    batch.check(stream=sh)
    batch.stats(reset=True)

    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    batch.check(stream=sh)
    stages = batch.stats(reset=True)
    launches = int(stages["kernel_launches"])  # this library's kernels in the timed region
    if not args.no_graph:
        # graph launches record no stage times: the breakdown comes from the
        # same steps launched one by one (CUDA events around each stage)
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                params.copy_(p_alt[k & 1], non_blocking=True)
                batch.set_params_dev(params, stream=sh)
                batch.forward_backward(img, data, sigma, chi2, grad, stream=sh)
        torch.cuda.synchronize()
        stages = batch.stats(reset=True)
    ms = max_over_ranks(world, ms)
    ms_per_step = ms / args.steps
    value = world * n_models * args.steps / (ms / 1000.0)
    pix_per_step = sum(w * h for (w, h) in batch.dims)

    # e2e through the public API with host buffers: parameters in from pinned
    # host memory, chi^2 and gradients back to pinned host memory, every step
    h_alt = [torch.tensor(par.ravel(), dtype=torch.float64).pin_memory(),
             torch.tensor(alt_np.ravel(), dtype=torch.float64).pin_memory()]
    h_par = h_alt[0]
    h_chi2 = torch.zeros(n_models, dtype=torch.float64).pin_memory()
    h_grad = torch.zeros(n_prof * 12, dtype=torch.float64).pin_memory()
    e2e_steps = max(3, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for _ in range(e2e_steps):
            params.copy_(h_alt[n_step[0] & 1], non_blocking=True)
            n_step[0] += 1
            if args.no_graph:
                batch.set_params_dev(params, stream=sh)
                batch.forward_backward(img, data, sigma, chi2, grad, stream=sh)
            else:
                batch.step_graph(params, img, data, sigma, chi2, grad, stream=sh)
            h_chi2.copy_(chi2, non_blocking=True)
            h_grad.copy_(grad, non_blocking=True)
            stream.synchronize()
    e2e_s = time.perf_counter() - t0
    e2e_value = world * n_models * e2e_steps / max_over_ranks(world, e2e_s)
    batch.stats(reset=True)

    # back to the parameters themselves for the counts and the accuracy checks
    with torch.cuda.stream(stream):
        params.copy_(p_alt[0], non_blocking=True)
        batch.set_params_dev(params, stream=sh)
        batch.forward_backward(img, data, sigma, chi2, grad, stream=sh)
    torch.cuda.synchronize()
    # evaluate_at calls per step (the tree's algorithmic work), from one
    # recorded forward pass
    batch.record_depth(True)
    with torch.cuda.stream(stream):
        batch.forward(img, stream=sh)
    torch.cuda.synchronize()
    counts = np.zeros(32)
    for _, c in batch.depth():
        counts += c
    batch.record_depth(False)
    evals = float(counts[30] + counts[31])

    # the plain FP64 per-model path (forward + VJP, one model per launch
    # sequence), timed on four models; on 32, its images, chi^2 and
    # gradients against the FP32 batch's (accuracy of the timed step)
    fp64_rates = []
    acc = {"flux": [], "pixel": [], "pixel3": [], "abs": [], "chi2": []}
    img32 = img.cpu().numpy()
    chi32 = chi2.cpu().numpy()
    grad32 = grad.cpu().numpy().reshape(n_prof, 12)
    first_prof = np.cumsum([0] + [len(s["profiles"]) for s in specs])
    n_acc = min(ACC_MODELS, n_models)
    g64_all, g32_all, im64_all = [], [], []
    if rank == 0:
        for i in range(n_acc):
            spec = specs[i]
            b1 = pg.Batch([W.to_model(spec, env64)], env64)
            b1.enable_adjoint()
            a, z = b1.offsets[0], b1.offsets[1]
            im1 = torch.zeros(z - a, dtype=torch.float64, device="cuda")
            d1 = torch.tensor(data_np[batch.offsets[i]:batch.offsets[i + 1]], dtype=torch.float64, device="cuda")
            s1 = torch.tensor(sigma_np[batch.offsets[i]:batch.offsets[i + 1]], dtype=torch.float64, device="cuda")
            c1 = torch.zeros(1, dtype=torch.float64, device="cuda")
            g1 = torch.zeros(len(spec["profiles"]) * 12, dtype=torch.float64, device="cuda")
            with torch.cuda.stream(stream):
                b1.forward_backward(im1, d1, s1, c1, g1, stream=sh)
            torch.cuda.synchronize()
            ref = im1.cpu().numpy()
            im64_all.append(ref)
            got = img32[batch.offsets[i]:batch.offsets[i + 1]].astype(np.float64)
            peak = np.abs(ref).max()
            bright = np.abs(ref) > 1e-9 * peak
            acc["pixel"].append(float(np.max(np.abs(got[bright] - ref[bright]) / np.abs(ref[bright]))))
            bright3 = np.abs(ref) > 1e-3 * peak
            acc["pixel3"].append(float(np.max(np.abs(got[bright3] - ref[bright3]) / np.abs(ref[bright3]))))
            acc["abs"].append(float(np.max(np.abs(got - ref)) / peak))
            acc["flux"].append(abs(got.sum() - ref.sum()) / abs(ref.sum()))
            acc["chi2"].append(abs(chi32[i] - c1.item()) / abs(c1.item()))
            g64_all.append(g1.cpu().numpy().reshape(-1, 12)[:, :8])
            g32_all.append(grad32[first_prof[i]:first_prof[i + 1], :8])
            if i >= 4:
                b1.close()
                continue
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            reps = 3
            with torch.cuda.stream(stream):
                for _ in range(reps):
                    b1.forward_backward(im1, d1, s1, c1, g1, stream=sh)
            e1.record(stream)
            torch.cuda.synchronize()
            fp64_rates.append(reps / (e0.elapsed_time(e1) / 1000.0))
            b1.close()
    grad_acc = None
    if rank == 0 and n_acc:
        grad_acc = gradient_accuracy(specs[:n_acc], par[:first_prof[n_acc]], np.concatenate(im64_all),
                                     data_np[:batch.offsets[n_acc]], sigma_np[:batch.offsets[n_acc]],
                                     np.concatenate(g32_all), np.concatenate(g64_all), env64)
    fp64_rate = statistics.median(fp64_rates) if fp64_rates else None

    # the same step with every convolution forced to the FFT, and to the
    # direct convolution (the autotuner picks per model by timing): models/s
    forced = {"fft": None, "brute": None}
    if rank == 0 and args.convolver == "auto" and not args.no_graph:
        for how in forced:
            models_f = [W.to_model(s, env32) for s in specs]
            for m in models_f:
                m.set_convolver(how)
            bf = pg.Batch(models_f, env32)
            bf.enable_adjoint()
            with torch.cuda.stream(stream):
                for k in range(2):
                    params.copy_(p_alt[k & 1], non_blocking=True)
                    bf.step_graph(params, img, data, sigma, chi2, grad, stream=sh)
            torch.cuda.synchronize()
            nf = max(3, args.steps // 2)
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            with torch.cuda.stream(stream):
                for k in range(nf):
                    params.copy_(p_alt[k & 1], non_blocking=True)
                    bf.step_graph(params, img, data, sigma, chi2, grad, stream=sh)
            f1.record(stream)
            torch.cuda.synchronize()
            bf.check(stream=sh)
            fms = f0.elapsed_time(f1) / nf
            forced[how] = {"value": n_models / (fms / 1000.0), "unit": "models/s", "ms_per_step": fms, "steps": nf}
            bf.close()

    if rank != 0:
        return

    # roofline of the dominant stage (stage times from CUDA events on the stream)
    per_step = {k: stages[k] / max(1, args.steps) for k in
                ("setup_ms", "eval_ms", "finish_ms", "chi2_ms", "adjoint_conv_ms", "backward_ms")}
    dom = max(per_step, key=per_step.get)
    sm_mhz = clk.get("sm_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s at the sampled clock
    # direct convolution: 2 flop per output pixel and PSF tap (forward over the
    # crop, adjoint over the drawing area)
    taps = [s["psf"].shape[0] * s["psf"].shape[1] for s in specs]
    conv_fwd = sum(2.0 * w * h * t for (w, h), t in zip(batch.dims, taps))
    conv_adj = sum(2.0 * (w + s["psf"].shape[1] // 2 * 2) * (h + s["psf"].shape[0] // 2 * 2) * t
                   for (w, h), t, s in zip(batch.dims, taps, specs))
    work = {"eval_ms": evals * FLOP_EVAL, "backward_ms": evals * FLOP_GRAD, "finish_ms": conv_fwd,
            "adjoint_conv_ms": conv_adj}
    # the FFT convolution (when the plan takes it for every model) is bound by
    # HBM: its algorithmic bytes per model (the three passes' reads and
    # writes, the PSF spectrum shared and read from L2), against the measured
    # copy bandwidth
    plan = batch.conv_info()
    fft_bytes = None
    if plan["fft_models"] == n_models:
        fwd_b = adj_b = 0.0
        for (cw, ch), s in zip(batch.dims, specs):
            kh, kw = s["psf"].shape
            dw, dh = cw + kw // 2 * 2, ch + kh // 2 * 2
            nb = fft_length(cw + kw) // 2 + 1
            # the direct canvas is read only where some profile is drawn unconvolved
            direct = any(not p.get("convolve", False) for _, p in s["profiles"])
            fwd_b += 4.0 * dw * dh + 16.0 * nb * (dh + ch) + (8.0 if direct else 4.0) * cw * ch
            adj_b += 4.0 * cw * ch + 16.0 * nb * (ch + dh) + 4.0 * dw * dh
        fft_bytes = {"finish_ms": fwd_b, "adjoint_conv_ms": adj_b}
    # DRAM bytes per launch, per model of this workload: ncu dram__bytes_read.sum +
    # dram__bytes_write.sum of each kernel on the 256-model copy of the workload
    # (one ncu capture per kernel), divided by 256
    traffic_per_model = {"eval_ms": 112.2e6 / 256, "backward_ms": 76.3e6 / 256, "finish_ms": 194.6e6 / 256,
                         "adjoint_conv_ms": ADJ_CONV_TRAFFIC_PER_MODEL}
    roof = {"bound": "fp32", "kernel": dom.replace("_ms", ""), "achieved": None, "peak": fp32_peak,
            "unit": "TFLOP/s", "frac": None, "traffic": None,
            "peak_note": "nominal FP32 FMA peak (152 SMs x 128 lanes x 2 flop) at the sampled median SM clock; "
                         "no measured FP32 peak exists for this pool"}
    if dom in work:
        achieved = work[dom] / (per_step[dom] / 1000.0) / 1e12
        tpm = traffic_per_model.get(dom)
        roof.update({"achieved": achieved, "frac": achieved / fp32_peak,
                     "traffic": tpm * n_models if tpm else None, "flop_per_step": work[dom]})
        if dom in ("eval_ms", "backward_ms"):
            roof.update({"evals_per_step": evals, "flop_per_eval": FLOP_EVAL if dom == "eval_ms" else FLOP_GRAD})
    # the same figures for each of the four large stages (which one dominates
    # changes with run-to-run noise: they are within ~6 % of each other)
    roof["by_kernel"] = {k.replace("_ms", ""): {"ms_per_step": per_step[k],
                                                "achieved": work[k] / (per_step[k] / 1000.0) / 1e12,
                                                "unit": "TFLOP/s",
                                                "frac": work[k] / (per_step[k] / 1000.0) / 1e12 / fp32_peak}
                         for k in work if per_step.get(k)}
    if fft_bytes:
        hbm = hbm_peak()
        for k, nbytes in fft_bytes.items():
            if per_step.get(k):
                gbs = nbytes / (per_step[k] / 1000.0) / 1e9
                roof["by_kernel"][k.replace("_ms", "")] = {
                    "ms_per_step": per_step[k], "method": "fft", "achieved": gbs, "unit": "GB/s",
                    "peak": hbm["gbs"], "peak_note": hbm["note"], "frac": gbs / hbm["gbs"],
                    "algorithmic_bytes_per_step": nbytes}
        if dom in fft_bytes:
            e = roof["by_kernel"][dom.replace("_ms", "")]
            roof.update({"bound": "hbm", "achieved": e["achieved"], "peak": e["peak"], "unit": "GB/s",
                         "frac": e["frac"], "traffic": None, "peak_note": e["peak_note"]})

    dropin = dropin_rates(env64, pg.get_cuda_environment(local, use_double=False)) if not args.no_dropin else None

    cpu = None
    if not args.no_cpu_baseline:
        v, threads, done, dt = cpu_baseline_sample(specs, par, budget_s=8.0)
        cpu = {"value": v, "unit": "models/s", "cores": threads, "kind": "port",
               "sample": "%d model(s) rendered + 33-point central-difference gradient in %.1f s" % (done, dt)}

    line = {
        "metric": METRIC, "value": value, "unit": "models/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "%d models 256x256, sersic bulge+disk, 25x25 Moffat PSF, model+VJP (chi2 + 16 "
                               "gradients per model)" % n_models, "models_per_gpu": n_models,
                   "pixels_per_model": 65536, "l2": "inputs larger than L2 (images+data %.0f MB)" %
                   (2 * 4 * pix_per_step / 1e6)},
        "mpix_per_s": world * pix_per_step * args.steps / (ms / 1000.0) / 1e6,
        "fp64_per_model_evals_per_s": fp64_rate,
        "accuracy": {"vs": "plain FP64 GPU path, same models and data (that path equals libprofit's CPU "
                           "result to 1e-10 per pixel)",
                     "models": len(acc["flux"]),
                     "max_rel_flux_err": max(acc["flux"]) if acc["flux"] else None,
                     "max_rel_pixel_err": max(acc["pixel"]) if acc["pixel"] else None,
                     "pixel_floor": "pixels above 1e-9 x the model's peak",
                     "max_rel_pixel_err_above_1e-3_peak": max(acc["pixel3"]) if acc["pixel3"] else None,
                     "max_abs_err_of_peak": max(acc["abs"]) if acc["abs"] else None,
                     "convolution": "FFT for %d of %d models (the FFT's rounding is absolute, relative to the "
                                    "peak: faint pixels carry it)" % (plan["fft_models"], n_models),
                     "max_rel_chi2_err": max(acc["chi2"]) if acc["chi2"] else None,
                     "grad": grad_acc},
        "fft_forced": forced["fft"],
        "direct_forced": forced["brute"],
        "drop_in": dropin,
        "ratio_vs_fp64_per_model": (value / world) / fp64_rate if fp64_rate else None,
        "stage_ms_per_step": per_step,
        "roofline": roof,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "models/s", "h2d_bytes_per_step": int(par.size * 8),
                "d2h_bytes_per_step": int(n_models * 8 + n_prof * 12 * 8)},
        # counted by the library: per step the parameter scatter, setup (solves, constants),
        # evaluation, convolution (direct and / or FFT passes), chi2, adjoint convolution,
        # backward, gradient reduction
        "gpu_launches": launches,
        "conv_plan": batch.conv_info(),
        "graph": not args.no_graph,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)

def run_workload(args, world, rank, local):
    """--workload cfg2 / cfg3 / cfg5 (module docstring)."""
    import torch
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    import workloads as W

    torch.cuda.set_device(local)
    env64 = pg.get_cuda_environment(local, use_double=True)
    env32 = pg.get_cuda_environment(local, use_double=False, profile=True)
    specs = W.cfg3(args.models or 4096) if args.workload == "cfg3" else W.CONFIGS[int(args.workload[3:])]()
    with_grad = args.workload == "cfg5"
    models = [W.to_model(s, env32) for s in specs]
    batch = pg.Batch(models, env32)
    img = torch.zeros(batch.total_pixels, dtype=torch.float32, device="cuda")
    n_models = len(specs)
    pix = sum(w * h for (w, h) in batch.dims)
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream
    if with_grad:
        batch.enable_adjoint()
        with torch.cuda.stream(stream):
            batch.forward(img, stream=sh)
        torch.cuda.synchronize()
        rng = np.random.Generator(np.random.PCG64(5000 + rank))
        ref = img.cpu().numpy().astype(np.float64)
        sig = 0.01 * np.abs(ref).max()
        data = torch.tensor(ref + rng.normal(0, sig, ref.shape), dtype=torch.float32, device="cuda")
        sigma = torch.full_like(data, sig)
        chi2 = torch.zeros(n_models, dtype=torch.float64, device="cuda")
        grad = torch.zeros(batch.n_profiles * 12, dtype=torch.float64, device="cuda")
    # consecutive steps alternate between the parameters and a copy moved by
    # ~1e-6 relative in every entry, as an optimiser's steps are
    par_w = W.param_matrix(specs)
    alt_w = par_w * (1 + 1e-6 * np.random.Generator(np.random.PCG64(6000 + rank)).standard_normal(par_w.shape))
    alt_w[:, 4] = np.minimum(alt_w[:, 4], 1.0)  # axrat stays <= 1
    p_alt = [torch.tensor(par_w.ravel(), dtype=torch.float64, device="cuda"),
             torch.tensor(alt_w.ravel(), dtype=torch.float64, device="cuda")]
    params = p_alt[0].clone()
    n_step = [0]

    def step():  # on `stream`
        params.copy_(p_alt[n_step[0] & 1], non_blocking=True)
        n_step[0] += 1
        if with_grad:
            batch.step_graph(params, img, data, sigma, chi2, grad, stream=sh)
        else:
            batch.set_params_dev(params, stream=sh)
            batch.forward(img, stream=sh)

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step()
    torch.cuda.synchronize()
    batch.check(stream=sh)
    batch.stats(reset=True)
    clocks = ClockSampler(local)
    clocks.start()
    barrier(world)
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            step()
    ev1.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    ms = max_over_ranks(world, ev0.elapsed_time(ev1))
    clk = clocks.stop()
    batch.check(stream=sh)
    stages = batch.stats(reset=True)
    launches = int(stages["kernel_launches"])
    if with_grad:  # stage breakdown from the same steps launched one by one
        with torch.cuda.stream(stream):
            for k in range(args.steps):
                params.copy_(p_alt[k & 1], non_blocking=True)
                batch.set_params_dev(params, stream=sh)
                batch.forward_backward(img, data, sigma, chi2, grad, stream=sh)
        torch.cuda.synchronize()
        stages = batch.stats(reset=True)
    per_step = {k: stages[k] / max(1, args.steps) for k in
                ("setup_ms", "eval_ms", "finish_ms", "chi2_ms", "adjoint_conv_ms", "backward_ms")}
    value = world * n_models * args.steps / (ms / 1000.0)

    # e2e through the public API: parameters in from pinned host memory, the
    # images (forward) or chi^2 and gradients (cfg5) back, every step
    h_alt = [torch.tensor(par_w.ravel(), dtype=torch.float64).pin_memory(),
             torch.tensor(alt_w.ravel(), dtype=torch.float64).pin_memory()]
    h_par = h_alt[0]
    d_par = torch.zeros_like(h_par, device="cuda")
    if with_grad:
        h_out = [torch.zeros(n_models, dtype=torch.float64).pin_memory(),
                 torch.zeros(batch.n_profiles * 12, dtype=torch.float64).pin_memory()]
        dev_out = [chi2, grad]
    else:
        h_out = [torch.zeros(batch.total_pixels, dtype=torch.float32).pin_memory()]
        dev_out = [img]
    e2e_steps = max(3, args.steps // 2)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    with torch.cuda.stream(stream):
        for k in range(e2e_steps):
            if with_grad:
                params.copy_(h_alt[k & 1], non_blocking=True)
                batch.step_graph(params, img, data, sigma, chi2, grad, stream=sh)
            else:
                d_par.copy_(h_alt[k & 1], non_blocking=True)
                batch.set_params_dev(d_par, stream=sh)
                batch.forward(img, stream=sh)
            for h, d in zip(h_out, dev_out):
                h.copy_(d, non_blocking=True)
            stream.synchronize()
    e2e_value = world * n_models * e2e_steps / max_over_ranks(world, time.perf_counter() - t0)
    if rank != 0:
        return
    # the image at the parameters themselves, for the accuracy check
    with torch.cuda.stream(stream):
        batch.set_params_dev(p_alt[0], stream=sh)
        batch.forward(img, stream=sh)
    torch.cuda.synchronize()

    # accuracy against the FP64 path on a sample of the models (cfg5: the
    # direct convolution, the FP64 FFT stopping at 4096 points)
    got = img.cpu().numpy().astype(np.float64)
    pick = list(range(n_models)) if n_models <= 4 else list(range(0, n_models, 64))
    models64 = [W.to_model(dict(specs[i], convolver="brute") if args.workload == "cfg5" else specs[i], env64)
                for i in pick]
    b64 = pg.Batch(models64, env64)
    img64 = torch.zeros(b64.total_pixels, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t64 = time.perf_counter()
    b64.forward(img64)
    b64.check()
    t64 = time.perf_counter() - t64
    o64 = img64.cpu().numpy()
    flux_err, pix_err, abs_err = [], [], []
    for j, i in enumerate(pick):
        a = got[batch.offsets[i]:batch.offsets[i + 1]]
        r = o64[b64.offsets[j]:b64.offsets[j + 1]]
        peak = np.abs(r).max()
        bright = np.abs(r) > 1e-3 * peak
        flux_err.append(abs(a.sum() - r.sum()) / abs(r.sum()))
        pix_err.append(float(np.max(np.abs(a[bright] - r[bright]) / np.abs(r[bright]))))
        abs_err.append(float(np.max(np.abs(a - r)) / peak))
    b64.close()

    cpu = None
    if not args.no_cpu_baseline and args.workload != "cfg5":
        from oracle import oracle as O
        O.build(with_ref=False)
        threads = os.cpu_count() or 1
        t0 = time.time()
        done = 0
        for spec in specs:
            O.evaluate(W.to_oracle_case(dict(spec, convolver="brute")), threads=threads)
            done += 1
            if time.time() - t0 > 8.0:
                break
        dt = time.time() - t0
        cpu = {"value": done / dt, "unit": "models/s", "cores": threads, "kind": "port",
               "sample": "%d model(s) rendered (direct convolution) in %.1f s" % (done, dt)}
    dom = max(per_step, key=per_step.get)
    desc = {"cfg2": "one 1000x1000 model: sersic bulge + disk + sky, 51x51 Moffat PSF by FFT, forward",
            "cfg3": "%d models, sides 64-512, 1-3 radial profiles of six kinds, own Moffat PSFs (15-41), "
                    "autotuned convolution, forward" % n_models,
            "cfg5": "one 4096x4096 field: 10,000 radial profiles + sky, 101x101 Moffat PSF by a 4608x4608 FFT, "
                    "forward + chi2 + gradients of all profiles"}[args.workload]
    line = {
        "metric": METRIC, "value": value, "unit": "models/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": desc, "models_per_gpu": n_models, "pixels": pix,
                   "l2": "inputs larger than L2" if pix * 4 > 129e6 else "inputs smaller than L2"},
        "mpix_per_s": world * pix * args.steps / (ms / 1000.0) / 1e6,
        "fp64_forward_s": t64, "fp64_models": len(pick),
        "accuracy": {"vs": "plain FP64 GPU path", "models": len(pick), "max_rel_flux_err": max(flux_err),
                     "max_rel_pixel_err": max(pix_err), "pixel_floor": "pixels above 1e-3 x the model's peak",
                     "max_abs_err_of_peak": max(abs_err)},
        "stage_ms_per_step": per_step,
        "roofline": {"bound": "fp32" if dom in ("eval_ms", "backward_ms") else "hbm", "kernel": dom[:-3],
                     "achieved": None, "peak": None, "unit": None, "frac": None, "traffic": None,
                     "note": "stage breakdown only; the per-kernel roofline is measured on the default workload"},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": "models/s", "h2d_bytes_per_step": int(h_par.numel() * 8),
                "d2h_bytes_per_step": int(sum(h.numel() * h.element_size() for h in h_out))},
        "gpu_launches": launches,
        "graph": with_grad,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)


def run_dropin(args, rank, local):
    """--workload dropin: the drop-in Model::evaluate path alone (cfg1 and
    cfg2 through pf_model_evaluate, host buffers in and out, one model per
    call, FP64 and FP32), with the CPU oracle port on the same models unless
    --no-cpu-baseline. value = cfg1's double-precision calls/s."""
    import __graft_entry__
    __graft_entry__.build_cuda()
    import libprofit_gb300 as pg
    if rank != 0:
        return
    env64 = pg.get_cuda_environment(local, use_double=True)
    env32 = pg.get_cuda_environment(local, use_double=False)
    clocks = ClockSampler(local)
    clocks.start()
    rates = dropin_rates(env64, env32, cpu=not args.no_cpu_baseline)
    clk = clocks.stop()
    line = {"metric": "drop-in Model::evaluate calls/s (one model per call, host buffers)",
            "value": rates["cfg1"]["fp64_calls_per_s"], "unit": "calls/s", "n_gpus": 1, "steps": None,
            "warmup": 3, "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "cfg1: one 100x100 sersic, 15x15 PSF, direct convolution (value); cfg2: one "
                                   "1000x1000 bulge + disk + sky, 51x51 PSF by FFT"},
            "drop_in": rates, "clocks": clk}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_init(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    elif args.workload == "dropin":
        run_dropin(args, rank, local)
    elif args.workload != "cfg4":
        run_workload(args, world, rank, local)
    else:
        run_ours(args, world, rank, local)
    if world > 1 and args.impl != "reference":
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
