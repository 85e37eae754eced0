"""Benchmark: converged Levenberg-Marquardt Sersic fits per second on one GB300,
learned + batched against plain.

Workloads (one "step" = every stamp of the workload fitted once, from its initial values):
  learned (default) -- 65,536 held-out 64 x 64 stamps rendered by this library: one Sersic
      galaxy from the C0 distributions + a flat sky of 1.0 (locked), Moffat PSF (beta 3.5,
      FWHM ~ U(2, 5) px, side 4 FWHM rounded to odd), Gaussian noise of constant sigma at
      SNR ~ U(10, 200).
      A step = CNN proposal (bf16 tensor-core kernels) + moments fallback, chi^2 of both,
      per-stamp selection, one batched LM of all stamps (7 free parameters), then LM's final
      chi^2 decides: stamps left more than 5 sigma above chi^2/ndf = 1 are fitted again by
      the plain method and keep the better fit.
      Reported beside it: the plain method = LM from the reference's own heuristic initial
      values (initialize(): centre of light, PA, isophote q, profile Nelder-Mead, computed by
      ap_reference_init), batched and one stamp at a time.
  init -- the reference's initial-value heuristics (initialize(), ap_reference_init) on the
      learned workload's stamps: stamps/s, parity and the CPU oracle beside it.
  livepsf -- fitted PSF models: 64 x 64 stamps of a compact Sersic galaxy convolved with a live
      Moffat PSF model on a 15 x 15 PSF image (set_aux_psf), PSF n and Rd fitted with the
      galaxy's 7 parameters by the scene LM one stamp after another (16 at a time on their own
      CUDA streams beside it): fits/s, parity and the CPU oracle beside it; plus
      200 galaxies on 1024 x 1024 sharing one live 31 x 31 Moffat PSF (1402 parameters) fitted
      jointly.
  cutouts -- N stamps (default 8192) with sides round(log-uniform(32, 256)) px, each one
      Sersic galaxy + a flat sky of 1.0 (locked), its own Moffat PSF (beta 3.5, FWHM ~
      U(2, 5) px, side = 4 FWHM rounded to odd), noise sigma = sqrt(model + 10), 7 free
      parameters from the truth perturbed by 10 %.
Rendering is FP32 with midpoint sampling + the reference's adaptive threshold integration,
bilinear sub-pixel PSF shift and PSF convolution; LM accumulators, damping solves and chi^2
are FP64.  Seeded synthetic data (no public dataset exists for this path).

Arms:
  default            the CUDA path (libastrophot_gb300.so) -- JSON line with value (device
                     resident inputs), e2e (host buffers, H2D + fit + D2H inside the timed
                     region), roofline of the dominant kernel, cpu_baseline, clocks.
  --impl reference   the reference algorithm's CPU implementation (the float64 restatement
                     in oracle/, pinned to the reference's outputs) on all host cores, on a
                     bounded sample of the same workload.
"""

from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

FREE_MASK = 0x7F  # cx cy q PA n Re Ie ; sky F locked


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="learned", choices=["learned", "cutouts", "crowded", "init", "livepsf"])
    p.add_argument("--stamps", type=int, default=None, help="65536 (learned, init) / 32 (livepsf) / 8192 (cutouts)")
    p.add_argument("--seed", type=int, default=2024)
    p.add_argument("--cpu-sample", type=int, default=None,
                   help="stamps fitted by the CPU oracle (parity + CPU baseline): 256 (learned, cutouts) / 8 (init, livepsf)")
    p.add_argument("--rounds-per-sync", type=int, default=8)
    p.add_argument("--grid", default=None,
                   help="blocks per SM of sample,integrate,conv,psf (default: the autotuner picks them)")
    p.add_argument("--livepsf-workers", type=int, default=16, help="concurrent fits (host threads / streams)")
    p.add_argument("--no-graph", action="store_true")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-crowded", action="store_true", help="skip the crowded-field block")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the single-stamp (128x128) and batched-cutout blocks of the default run")
    p.add_argument("--no-cnn", action="store_true", help="skip the CNN inference / training block")
    p.add_argument("--c0-stamps", type=int, default=64, help="seeds of the 128x128 single-stamp block")
    p.add_argument("--c0-cpu-sample", type=int, default=32, help="of them fitted by the oracle")
    p.add_argument("--cutout-stamps", type=int, default=8192, help="stamps of the batched-cutout block")
    p.add_argument("--cutout-cpu-sample", type=int, default=64, help="of them fitted by the oracle")
    p.add_argument("--crowded-size", type=int, default=1024)
    p.add_argument("--crowded-sources", type=int, default=200)
    p.add_argument("--crowded-iters", type=int, default=20)
    a = p.parse_args()
    if a.stamps is None:
        a.stamps = 65536 if a.workload in ("learned", "init") else (32 if a.workload == "livepsf" else 8192)
    return a


def rank_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


# ----------------------------------------------------------------------------------------
# workload
# ----------------------------------------------------------------------------------------


def workload_specs(n, seed, rank=0):
    from astrophot_gb300 import synthetic

    return synthetic.cutout_stamps(n, seed + 7919 * rank)


def truth_and_init_rows(specs):
    truth = np.array([np.r_[s.truth, 0.0] for s in specs])
    init = np.array([np.r_[s.init, 0.0] for s in specs])
    return truth, init


def sample_indices(specs, k):
    """k stamps spread over the size distribution (sorted by area, evenly spaced)."""
    order = np.argsort([s.nx * s.ny for s in specs], kind="stable")
    if k >= len(specs):
        return list(order)
    pick = np.linspace(0, len(specs) - 1, k).round().astype(int)
    return [int(order[i]) for i in pick]


# ----------------------------------------------------------------------------------------
# CPU side (oracle = float64 restatement of the reference algorithm)
# ----------------------------------------------------------------------------------------


def _oracle_fit(args):
    """One fit with the oracle: (data, weight, psf, init8, truth8) -> (chi2, iters, seconds).
    Without init8 the fit starts from the reference's own ``initialize()`` heuristics (restated
    in float64), as a reference user's fit does."""
    data, weight, psf, init, _ = args
    from oracle.lm import GroupProblem, LMOracle
    from oracle.render import PSF, Component, Window

    if init is None:
        from oracle.refinit import initialize

        o = initialize(data, "sersic", 1.0)
        init = (o["center"][0], o["center"][1], o["q"], o["PA"], o["n"], o["Re"], o["Ie"], 0.0)
    cx, cy, q, PA, n, Re, Ie, F = init
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
    sky = Component("flat_sky", {"F": F}, locked=("F",))
    ny, nx = data.shape
    prob = GroupProblem([gal, sky], Window.from_scale(nx, ny), PSF(psf), data, weight)
    t = time.perf_counter()
    lm = LMOracle(prob, prob.representation()).fit()
    return lm.res_loss(), lm.iterations, time.perf_counter() - t, lm.message


def _oracle_fit_full(args, knobs=None):
    """:func:`_oracle_fit` plus the fitted value-space vector: (chi2, iters, seconds, message,
    values[8]); ``knobs`` are the galaxy's sampling knobs (default: the reference's)."""
    data, weight, psf, init, _ = args
    from oracle.lm import GroupProblem, LMOracle
    from oracle.render import PSF, Component, Window

    cx, cy, q, PA, n, Re, Ie, F = init
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full",
                    **(knobs or {}))
    sky = Component("flat_sky", {"F": F}, locked=("F",))
    ny, nx = data.shape
    prob = GroupProblem([gal, sky], Window.from_scale(nx, ny), PSF(psf), data, weight)
    t = time.perf_counter()
    lm = LMOracle(prob, prob.representation()).fit()
    sec = time.perf_counter() - t
    from astrophot_gb300.transforms import rep_to_slots

    vals = rep_to_slots(lm.res()[None, :], np.asarray(init, dtype=np.float64)[None, :], FREE_MASK)[0]
    return lm.res_loss(), lm.iterations, sec, lm.message, vals


def value_rel_diff(got, ref):
    """Relative difference of fitted value-space vectors [cx, cy, q, PA, n, Re, Ie]: |d| / |ref|,
    except PA, whose difference is taken modulo pi (the same orientation) and divided by pi, and
    Ie (log10 of the brightness), compared as the relative difference of the brightness
    10^Ie, |d Ie| ln 10."""
    got, ref = np.asarray(got, dtype=np.float64)[:7], np.asarray(ref, dtype=np.float64)[:7]
    d = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-300)
    dpa = (got[3] - ref[3] + np.pi / 2) % np.pi - np.pi / 2
    d[3] = abs(dpa) / np.pi
    d[6] = abs(got[6] - ref[6]) * math.log(10.0)
    return d


def oracle_parity(jobs, gpu_chi2, gpu_values, gpu_messages, processes, fit=None):
    """The float64 oracle LM on ``jobs`` (same data and initial values as the GPU fits) in a
    spawned process pool: the CPU baseline (fits/s on ``processes`` cores) and the parity of the
    GPU fits -- chi^2 within 1e-4 relative, the same message, fitted parameters within 1e-4."""
    fit = fit or _oracle_fit_full
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes=processes) as pool:
        pool.map(fit, jobs[: min(len(jobs), processes)])  # imports, warm caches
        t = time.perf_counter()
        res = pool.map(fit, jobs)
        wall = time.perf_counter() - t
    rel_c = np.array([abs(g / r[0] - 1.0) for g, r in zip(gpu_chi2, res)])
    dv = np.array([value_rel_diff(gv, r[4]) for gv, r in zip(gpu_values, res)])
    rel_v = dv.max(axis=1)
    same = np.array([gm == r[3] for gm, r in zip(gpu_messages, res)])
    ostat, gstat = {}, {}
    for gm, r in zip(gpu_messages, res):
        ostat[r[3]] = ostat.get(r[3], 0) + 1
        gstat[gm] = gstat.get(gm, 0) + 1
    parity = {
        "stamps": len(jobs),
        "within_1e-4": int(np.sum(rel_c <= 1e-4)),
        "max_rel_chi2_vs_oracle": float(rel_c.max()),
        "same_message": int(same.sum()),
        "params_within_1e-4": int(np.sum(rel_v <= 1e-4)),
        "max_rel_params_vs_oracle": float(rel_v.max()),
        "params_rel_p99": float(np.quantile(rel_v, 0.99)),
        # the fits beyond 1e-4: which parameter, and the axis ratio the oracle fitted (near 1 the
        # position angle is undetermined and moves with any rounding)
        "params_outliers": [{"param": ["cx", "cy", "q", "PA", "n", "Re", "Ie"][int(np.argmax(dv[k]))],
                             "rel": float(rel_v[k]), "oracle_q": float(res[k][4][2])}
                            for k in np.flatnonzero(rel_v > 1e-4)[:8]],
        "oracle_messages": ostat,
        "gpu_messages": gstat,
        "oracle_mean_iterations": float(np.mean([r[1] for r in res])),
        "params_rule": "value-space [cx, cy, q, PA, n, Re, Ie], |d| / |ref|; PA difference modulo pi over pi; "
                       "Ie as the relative brightness |d Ie| ln 10",
    }
    cpu = {"value": len(jobs) / wall, "unit": "fits/s", "cores": processes, "kind": "port"}
    return parity, cpu


def oracle_truth_image(spec):
    from oracle.render import PSF, Component, Window, sample_group

    cx, cy, q, PA, n, Re, Ie = spec.truth
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
    sky = Component("flat_sky", {"F": 0.0}, locked=("F",))
    model, _ = sample_group([gal, sky], Window.from_scale(spec.nx, spec.ny), PSF(spec.psf))
    return model


def run_reference(args):
    """--impl reference: the oracle LM over all host cores on a bounded sample."""
    from astrophot_gb300 import synthetic

    rank, world, _ = rank_info()
    if rank != 0:
        return
    specs = workload_specs(args.stamps, args.seed)
    cores = os.cpu_count() or 1
    idx = sample_indices(specs, max(cores, 1))
    jobs = []
    for i in idx:
        s = specs[i]
        truth = oracle_truth_image(s)
        data, weight = synthetic.add_noise(truth, s.seed)
        jobs.append((data, weight, s.psf, np.r_[s.init, 0.0], np.r_[s.truth, 0.0]))
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes=min(cores, len(jobs))) as pool:
        for _ in range(max(args.warmup, 0) and 1):
            pool.map(_oracle_fit, jobs[: min(len(jobs), cores)])
        times = []
        for _ in range(args.steps):
            t = time.perf_counter()
            res = pool.map(_oracle_fit, jobs)
            times.append(time.perf_counter() - t)
    dt = statistics.median(times)
    value = len(jobs) / dt
    line = {
        "impl": "reference",
        "metric": "LM Sersic fits/s (chi2 within 1e-4 of the FP64 oracle)",
        "value": value,
        "unit": "fits/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {
            "workload": f"batched cutouts: {args.stamps} stamps 32-256 px, Sersic + sky, Moffat 9-21 px PSF",
            "sample": f"{len(jobs)} stamps spread over the size distribution, one per core",
        },
        "cpu_baseline": {
            "value": value,
            "unit": "fits/s",
            "cores": min(cores, len(jobs)),
            "kind": "port",
            "sample": f"{len(jobs)} stamps (float64 numpy restatement of the reference LM)",
        },
        "e2e": {"value": value, "unit": "fits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "mean_iterations": float(np.mean([r[1] for r in res])),
    }
    print(json.dumps(line), flush=True)


def aggregate_ranks(dev_ms, e2e_ms, converged, total, device):
    """Max of the per-rank times, sum of the per-rank fit counts (independent stamps per rank:
    weak scaling, no data-path collective; this is the only cross-rank step)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return dev_ms, e2e_ms, converged, total
    t = torch.tensor([dev_ms, e2e_ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    c = torch.tensor([converged, total], dtype=torch.float64, device=device)
    dist.all_reduce(c)
    return float(t[0]), float(t[1]), int(c[0]), int(c[1])


# ----------------------------------------------------------------------------------------
# GPU side
# ----------------------------------------------------------------------------------------


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = (
        "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, index=0):
        self.index = index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE,
                stderr=subprocess.DEVNULL,
                text=True,
            )
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                out, _ = self.proc.communicate()
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            parts = [p.strip() for p in l.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for name, v in zip(names, parts[4:8]):
                if v.lower() in ("active", "1"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons), "samples": len(sm)}


def run_gpu(args):
    if args.workload == "learned":
        run_gpu_learned(args)
    elif args.workload == "init":
        run_gpu_init(args)
    elif args.workload == "livepsf":
        run_gpu_livepsf(args)
    elif args.workload == "crowded":
        import torch

        if rank_info()[0] == 0:
            dev = torch.device("cuda")
            line = {"workload": "crowded", "crowded_field": crowded_block(args, dev)}
            if not args.no_configs:
                line["bulge_disk_field"] = bulge_disk_block(args, dev)
            print(json.dumps(line), flush=True)
    else:
        run_gpu_cutouts(args)


def run_gpu_cutouts(args):
    import torch

    from astrophot_gb300 import _native as N
    from astrophot_gb300 import synthetic
    from astrophot_gb300.transforms import slots_to_rep

    rank, world, local = rank_info()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())

    # every rank fits its own independent stamps (weak scaling, no data-path collective)
    specs = workload_specs(args.stamps, args.seed, rank)
    S = len(specs)
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=FREE_MASK, has_sky=True)
    batch = N.StampBatch(
        [(s.nx, s.ny) for s in specs], [(s.psf.shape[1], s.psf.shape[0]) for s in specs], N.scale_geometry(S), opts, dev
    )
    truth, init = truth_and_init_rows(specs)
    psf_h = np.concatenate([s.psf.astype(np.float32).ravel() for s in specs])
    psf_d = torch.from_numpy(psf_h).to(dev)
    model = batch.render(torch.from_numpy(truth).to(dev), psf_d)
    models = batch.unpack(model)
    data_l, w_l = [], []
    for s, m in zip(specs, models):
        d, w = synthetic.add_noise(m.astype(np.float64), s.seed)
        data_l.append(d.astype(np.float32).ravel())
        w_l.append(w.astype(np.float32).ravel())
    data_h = torch.from_numpy(np.concatenate(data_l)).pin_memory()
    weight_h = torch.from_numpy(np.concatenate(w_l)).pin_memory()
    psf_hp = torch.from_numpy(psf_h).pin_memory()
    fixed_h = torch.from_numpy(init).pin_memory()
    state0_h = torch.from_numpy(slots_to_rep(init, FREE_MASK)).pin_memory()
    data_d = data_h.to(dev)
    weight_d = weight_h.to(dev)
    fixed_d = fixed_h.to(dev)
    state0_d = state0_h.to(dev)
    lmo = N.make_lm_options(rounds_per_sync=args.rounds_per_sync, use_graph=not args.no_graph)

    def step_device():
        return batch.lm_fit(data_d, weight_d, None, psf_d, fixed_d, state0_d, lmo)

    for _ in range(max(args.warmup, 0)):
        step_device()
    torch.cuda.synchronize()

    # ---- value: inputs resident in HBM -------------------------------------------------
    batch.profile(True)
    batch.work_counters(reset=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    results = []
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            results.append(step_device())
        e1.record()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    dev_ms = e0.elapsed_time(e1) / args.steps
    ktimes = batch.kernel_times()
    work = batch.work_counters(reset=True)
    batch.profile(False)
    state, chi2, iters, status = results[-1]
    status_h = status.cpu().numpy()
    iters_h = iters.cpu().numpy()
    chi2_h = chi2.cpu().numpy()
    converged = int(np.sum((status_h == N.LM_SUCCESS) | (status_h == N.LM_IMMOBILE)))

    # ---- e2e: host buffers, copies inside the timed region -------------------------------
    def step_e2e():
        d = data_h.to(dev, non_blocking=True)
        w = weight_h.to(dev, non_blocking=True)
        p = psf_hp.to(dev, non_blocking=True)
        f = fixed_h.to(dev, non_blocking=True)
        s0 = state0_h.to(dev, non_blocking=True)
        st, c2, it, stt = batch.lm_fit(d, w, None, p, f, s0, lmo)
        return st.cpu(), c2.cpu(), stt.cpu()

    step_e2e()
    torch.cuda.synchronize()
    h2d = (data_h.numel() + weight_h.numel() + psf_hp.numel()) * 4 + (fixed_h.numel() + state0_h.numel()) * 8
    d2h = state.numel() * 8 + chi2.numel() * 8 + status.numel() * 4
    t0 = time.perf_counter()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    e2.record()
    for _ in range(args.steps):
        step_e2e()
    e3.record()
    torch.cuda.synchronize()
    e2e_ms = e2.elapsed_time(e3) / args.steps
    e2e_wall_ms = (time.perf_counter() - t0) * 1e3 / args.steps

    # max over ranks
    dev_ms, e2e_ms, converged_all, total_all = aggregate_ranks(dev_ms, e2e_ms, converged, S, dev)

    # ---- roofline of the dominant kernel (live CUDA-event times over the timed region) ----
    dominant = max(ktimes, key=lambda k: ktimes[k][0])
    fp32_peak = N.fma_probe_tflops()
    conv_ms, conv_n = ktimes["conv"]
    roof = None
    if dominant == "conv" and conv_ms > 0:
        achieved = work["conv_flops"] / (conv_ms * 1e-3) / 1e12
        roof = {
            "kernel": "k_conv (PSF convolution + fused Jacobian/chi2/JtWJ/JtWr)",
            "bound": "fp32",
            "achieved": achieved,
            "peak": fp32_peak,
            "unit": "TFLOP/s",
            "frac": achieved / fp32_peak,
            "traffic": None,
            "launches": conv_n,
            "avg_launch_ms": conv_ms / max(conv_n, 1),
            "peak_source": "measured FP32 FMA probe (ap_fma_probe) on this GPU",
        }
    else:
        ms, n = ktimes[dominant]
        roof = {"kernel": dominant, "bound": "fp32", "achieved": None, "peak": fp32_peak, "unit": "TFLOP/s",
                "frac": None, "traffic": None, "launches": n, "avg_launch_ms": ms / max(n, 1)}

    line = {
        "metric": "LM Sersic fits/s (chi2 within 1e-4 of the FP64 oracle)",
        "value": converged_all / (dev_ms * 1e-3),
        "unit": "fits/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 render / f64 LM",
        "data": "synthetic",
        "config": {
            "workload": f"batched cutouts: {S} stamps per GPU, sides log-uniform 32-256 px, Sersic + locked sky, "
            "Moffat PSF 9-21 px, 7 free params, midpoint + threshold integration, bilinear PSF shift",
            "stamps_per_gpu": S,
            "pixels_per_gpu": int(batch.out_pixels),
            "parallelism": f"replicas x{world} (independent stamps per rank)",
            "l2": "inputs (%.2f GB) exceed the 129 MB L2" % ((data_h.numel() + weight_h.numel()) * 4 / 1e9),
            "rounds_per_sync": args.rounds_per_sync,
            "cuda_graph": not args.no_graph,
        },
        "fits": {"total": int(total_all), "converged": int(converged_all),
                 "mean_iterations": float(iters_h.mean()),
                 "status_counts": {N.LM_MESSAGES[k]: int(np.sum(status_h == k)) for k in np.unique(status_h)}},
        "clocks": clk.summary(),
        "e2e": {"value": converged_all / (e2e_ms * 1e-3), "unit": "fits/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "wall_ms_per_step": e2e_wall_ms},
        "roofline": roof,
        "kernel_ms_per_step": {k: v[0] / args.steps for k, v in ktimes.items()},
        "kernel_launches_per_step": {k: v[1] / args.steps for k, v in ktimes.items()},
        "gpu_launches": int(sum(v[1] for v in ktimes.values()) / args.steps),
        "work_per_step": {k: v / args.steps for k, v in work.items()},
    }

    # ---- CPU baseline + parity on a bounded sample (rank 0, N = 1 only) -------------------
    if rank == 0 and world == 1 and not args.no_cpu and args.cpu_sample > 0:
        from astrophot_gb300.transforms import rep_to_slots

        idx = sample_indices(specs, args.cpu_sample)
        st_h = state.cpu().numpy()
        vals_h = rep_to_slots(st_h, init, FREE_MASK)
        jobs = []
        for i in idx:
            s = specs[i]
            o = batch.out_offsets[i]
            d = data_h[o : o + s.nx * s.ny].numpy().astype(np.float64).reshape(s.ny, s.nx)
            w = weight_h[o : o + s.nx * s.ny].numpy().astype(np.float64).reshape(s.ny, s.nx)
            jobs.append((d, w, s.psf.astype(np.float32).astype(np.float64), init[i], truth[i]))
        procs = max(1, min(os.cpu_count() or 1, len(jobs)))
        parity, cpu = oracle_parity(jobs, [chi2_h[i] for i in idx], [vals_h[i] for i in idx],
                                    [N.LM_MESSAGES[int(status_h[i])] for i in idx], procs)
        cpu["sample"] = (f"{len(idx)} stamps of this workload spread over the size range, from the same initial "
                         f"values; float64 numpy restatement of the reference LM on {procs} host processes")
        line["cpu_baseline"] = cpu
        line["parity"] = parity
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ----------------------------------------------------------------------------------------
# learned + batched workload
# ----------------------------------------------------------------------------------------


def learned_sample_jobs(S, seed, idx, data_of=None, init_of=None):
    """Oracle LM jobs for stamps ``idx`` of the learned workload.  ``data_of(i)`` gives the
    (data, sigma) the GPU fitted; without it the stamp is re-rendered by the oracle with
    numpy noise of the same sigma rule (same truth, PSF and SNR draws as the GPU's).
    ``init_of(i)`` gives the initial values; without it the fit starts from the reference's
    ``initialize()`` heuristics, computed inside the timed worker."""
    from astrophot_gb300 import cnn
    from oracle.render import PSF, Component, Window, sample_group

    rng = np.random.default_rng(seed)
    truth = cnn.draw_stamp_params(rng, S)
    pidx = rng.integers(0, 64, S)
    snr = rng.uniform(10.0, 200.0, S)
    bank = [k.astype(np.float32).astype(np.float64) for k in cnn.psf_bank()]
    jobs = []
    for i in idx:
        psf = bank[pidx[i]]
        if data_of is not None:
            data, sigma = data_of(i)
        else:
            cx, cy, q, PA, n, Re, Ie, F = truth[i]
            gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie},
                            psf_mode="full")
            sky = Component("flat_sky", {"F": 0.0}, locked=("F",))
            model, _ = sample_group([gal, sky], Window.from_scale(64, 64), PSF(psf))
            sigma = math.sqrt(np.sum((model - 1.0) ** 2)) / snr[i]
            data = model + sigma * np.random.default_rng(seed * 7919 + 17 + int(i)).normal(size=model.shape)
        weight = np.full(data.shape, 1.0 / sigma**2)
        init = init_of(i) if init_of is not None else None  # None: the worker runs initialize()
        jobs.append((data, weight, psf, init, truth[i]))
    return jobs


def run_reference_learned(args):
    """--impl reference, learned workload: the plain method on the CPU (the reference's
    ``initialize()`` heuristics, then its LM, both restated in float64) over all host cores on a
    bounded sample."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    k = min(args.stamps, 2 * cores)
    idx = list(np.linspace(0, args.stamps - 1, k).round().astype(int))
    jobs = learned_sample_jobs(args.stamps, args.seed, idx)
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes=min(cores, len(jobs))) as pool:
        if args.warmup > 0:
            pool.map(_oracle_fit, jobs[: min(len(jobs), cores)])
        times = []
        for _ in range(args.steps):
            t = time.perf_counter()
            res = pool.map(_oracle_fit, jobs)
            times.append(time.perf_counter() - t)
    dt = statistics.median(times)
    value = len(jobs) / dt
    line = {
        "impl": "reference",
        "metric": "LM Sersic fits/s (chi2 within 1e-4 of the FP64 oracle), learned+batched vs plain",
        "value": value,
        "unit": "fits/s",
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dt * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {
            "workload": f"learned init: {args.stamps} held-out 64x64 Sersic stamps + sky, Moffat FWHM 2-5 px, "
            "SNR 10-200; plain method (the reference's initialize() heuristics, then float64 LM)",
            "sample": f"{len(jobs)} stamps evenly spaced over the workload, {min(cores, len(jobs))} processes",
        },
        "cpu_baseline": {
            "value": value,
            "unit": "fits/s",
            "cores": min(cores, len(jobs)),
            "kind": "port",
            "sample": f"{len(jobs)} stamps (float64 numpy restatement of the reference initialize() + LM)",
        },
        "e2e": {"value": value, "unit": "fits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "mean_iterations": float(np.mean([r[1] for r in res])),
    }
    print(json.dumps(line), flush=True)


# kernels of this library launched per CNN proposal chunk: prepare, input im2col, 3 im2col,
# 6 GEMMs, 6 bias/activation passes, decode
CNN_LAUNCHES_PER_CHUNK = 18


def run_gpu_learned(args):
    import torch

    from astrophot_gb300 import _native as N
    from astrophot_gb300 import cnn

    rank, world, local = rank_info()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    S = args.stamps
    seed = args.seed + 7919 * rank
    st = cnn.make_stamps(S, seed, device=dev)
    net = cnn.InitNet.load(device=dev)
    lmo = N.make_lm_options(rounds_per_sync=args.rounds_per_sync, use_graph=not args.no_graph)
    batch = st.batch
    data_h = st.data.cpu().pin_memory()
    weight_h = st.weight.cpu().pin_memory()
    psf_h = st.psf.cpu().pin_memory()
    sigma_h = st.sigma.cpu().pin_memory()

    # in-project autotuners (outside the timed region): CNN GEMM tile shapes per layer shape,
    # persistent-grid sizes of the render pass
    N.lib().ap_cnn_autotune(1, None)
    if args.grid:
        grid = dict(zip(N.StampBatch.GRID_KNOBS, (int(v) for v in args.grid.split(","))))
        batch.set_grid(grid)
        tuned = {"blocks_per_sm": grid, "render_pass_ms": None, "fixed": True}
    else:
        tuned = batch.autotune(cnn.moments_init(st, S), st.psf, jacobian=True)

    def step_device():
        return cnn.learned_fit(net, st, S, lmo)

    def step_plain():
        return cnn.plain_fit(st, S, lmo)

    for _ in range(max(args.warmup, 0)):
        step_device()
    step_plain()
    torch.cuda.synchronize()

    # ---- value: learned + batched, inputs resident in HBM --------------------------------
    batch.profile(True)
    batch.work_counters(reset=True)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    results = []
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            results.append(step_device())
        e1.record()
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    dev_ms = e0.elapsed_time(e1) / args.steps
    ktimes = batch.kernel_times()
    work = batch.work_counters(reset=True)
    batch.profile(False)
    init_l, which, (state, chi2, iters, status) = results[-1]
    status_h, iters_h, chi2_h = status.cpu().numpy(), iters.cpu().numpy(), chi2.cpu().numpy()
    converged = int(np.sum((status_h == N.LM_SUCCESS) | (status_h == N.LM_IMMOBILE)))

    # ---- plain method on the GPU: the reference's heuristic values, batched and one stamp at
    # a time (the heuristic initialiser is inside the timed region) ----------------------------
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        init_p, (st_p, c2_p, it_p, stat_p) = step_plain()
    e1.record()
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / args.steps
    e0.record()
    cnn.heuristic_init(st, S)
    e1.record()
    torch.cuda.synchronize()
    heur_ms = e0.elapsed_time(e1)
    stat_ph = stat_p.cpu().numpy()
    conv_p = int(np.sum((stat_ph == N.LM_SUCCESS) | (stat_ph == N.LM_IMMOBILE)))
    n_single = min(32, S)
    init_ph = init_p.cpu()
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=FREE_MASK, has_sky=True)
    singles = []
    psf_off = [0]
    for kx, ky in batch.psf_shapes:
        psf_off.append(psf_off[-1] + kx * ky)
    for i in range(n_single):
        sl = slice(i * 4096, (i + 1) * 4096)
        one = N.StampBatch([(64, 64)], [batch.psf_shapes[i]], N.scale_geometry(1), opts, dev)
        singles.append(cnn.StampSet(st.truth[i : i + 1], st.data[sl].contiguous(), st.weight[sl].contiguous(),
                                    st.psf[psf_off[i] : psf_off[i + 1]].contiguous(), st.sigma[i : i + 1].contiguous(),
                                    one))
    cnn._lm(singles[0], init_p[0:1].contiguous(), lmo)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    conv_single = 0
    for i, ss in enumerate(singles):
        ini = cnn.heuristic_init(ss, 1)
        _, _, _, stt = cnn._lm(ss, ini, lmo)
        conv_single += int(stt.item() in (N.LM_SUCCESS, N.LM_IMMOBILE))
    torch.cuda.synchronize()
    single_s = time.perf_counter() - t0

    # ---- e2e: host buffers, copies inside the timed region -------------------------------
    # every step's inputs go from pinned host memory to the device through the public
    # learned_fit_host, which uploads the next batch on a copy stream while the current one is
    # fitted; the fitted state, chi^2 and status come back to the host every step
    host_in = (data_h, weight_h, psf_h, sigma_h)

    def run_e2e(steps):
        for _ in cnn.learned_fit_host(net, (host_in for _ in range(steps)), batch, S, lmo):
            pass

    run_e2e(2)
    torch.cuda.synchronize()
    h2d = (data_h.numel() + weight_h.numel() + psf_h.numel() + sigma_h.numel()) * 4
    d2h = state.numel() * 8 + chi2.numel() * 8 + iters.numel() * 4 + status.numel() * 4
    t0 = time.perf_counter()
    e0.record()
    run_e2e(args.steps)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e2e_wall_ms = (time.perf_counter() - t0) * 1e3 / args.steps

    dev_ms, e2e_ms, converged_all, total_all = aggregate_ranks(dev_ms, e2e_ms, converged, S, dev)

    fp32_peak = N.fma_probe_tflops()
    conv_ms, conv_n = ktimes["conv"]
    achieved = work["conv_flops"] / (conv_ms * 1e-3) / 1e12 if conv_ms > 0 else None
    roof = {
        "kernel": "k_conv (PSF convolution + fused Jacobian/chi2/JtWJ/JtWr)",
        "bound": "fp32",
        "achieved": achieved,
        "peak": fp32_peak,
        "unit": "TFLOP/s",
        "frac": achieved / fp32_peak if achieved else None,
        # DRAM bytes per launch from an ncu capture of three LM-round launches of the 4096-stamp
        # case (30.3 MB each on average, reads + writes), scaled by the stamps per launch
        "traffic": 30.3e6 * S / 4096,
        "traffic_unit": "bytes per launch (ncu, 4096-stamp capture scaled by stamps)",
        "launches": conv_n,
        "avg_launch_ms": conv_ms / max(conv_n, 1),
        "algorithmic_flop_per_launch": work["conv_flops"] / max(conv_n, 1),
        "peak_source": "measured FP32 FMA probe (ap_fma_probe) on this GPU",
    }
    # the adaptive integration (k_level1, its float64 re-decisions, k_integrate): samples of each
    # kind of evaluation against the rate of the same sample arithmetic alone (ap_sample_probe)
    integ_ms = ktimes["integrate"][0]
    n_all, n_diff, n_jac = work["integrate_samples"], work["integrate_samples_diff"], work["integrate_samples_jacobian"]
    rates = {k: N.sample_probe_rate(k) for k in (0, 1, 2)}
    ideal_s = (n_all - n_diff - n_jac) / rates[0] + n_jac / rates[1] + n_diff / rates[2]
    roof_int = {
        "kernel": "k_level1 + k_level1_amb + k_integrate (adaptive sub-pixel integration)",
        "bound": "sample arithmetic (FP32 + MUFU pipes)",
        "achieved": n_all / (integ_ms * 1e-3) / 1e9 if integ_ms > 0 else None,
        "peak": n_all / ideal_s / 1e9 if ideal_s > 0 else None,
        "unit": "Gsamples/s",
        "frac": ideal_s / (integ_ms * 1e-3) if integ_ms > 0 else None,
        "samples_per_step": {"all": n_all / args.steps, "difference": n_diff / args.steps,
                             "jacobian": n_jac / args.steps},
        "peak_source": "measured: the integration's own sample functions, register-resident at full occupancy "
                       "(ap_sample_probe: %.1f / %.1f / %.1f Gsamples/s plain / with partials / difference), "
                       "mixed by the counted samples" % (rates[0] / 1e9, rates[1] / 1e9, rates[2] / 1e9),
    }
    chunks = (S + 8191) // 8192
    launches = int(sum(v[1] for v in ktimes.values()) / args.steps) + CNN_LAUNCHES_PER_CHUNK * chunks + 2
    value = converged_all / (dev_ms * 1e-3)
    single_rate = conv_single / single_s if single_s > 0 else None
    line = {
        "metric": "LM Sersic fits/s (chi2 within 1e-4 of the FP64 oracle), learned+batched vs plain",
        "value": value,
        "unit": "fits/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 render / f64 LM / bf16 CNN",
        "data": "synthetic",
        "config": {
            "workload": f"learned init + batched LM: {S} held-out 64x64 stamps per GPU, Sersic (C0 distributions) "
            "+ locked sky 1.0, Moffat FWHM U(2,5) px of side odd(4 FWHM) = 9-21 px, SNR U(10,200); 7 free params",
            "stamps_per_gpu": S,
            "pixels_per_gpu": int(batch.out_pixels),
            "parallelism": f"replicas x{world} (independent stamps per rank)",
            "l2": "inputs (%.2f GB) exceed the 129 MB L2" % ((data_h.numel() + weight_h.numel()) * 4 / 1e9),
            "rounds_per_sync": args.rounds_per_sync,
            "cuda_graph": not args.no_graph,
        },
        "fits": {"total": int(total_all), "converged": int(converged_all),
                 "proposal_used": float(np.mean(which.cpu().numpy() == 0)),
                 "plain_refits": int(np.sum(which.cpu().numpy() == 2)),
                 "mean_iterations": float(iters_h.mean()),
                 "status_counts": {N.LM_MESSAGES[k]: int(np.sum(status_h == k)) for k in np.unique(status_h)}},
        "plain": {
            "batched_fits_per_s": conv_p / (plain_ms * 1e-3),
            "batched_ms_per_step": plain_ms,
            "heuristic_init_ms": heur_ms,
            "batched_mean_iterations": float(it_p.cpu().numpy().mean()),
            "batched_converged": conv_p,
            "single_fits_per_s": single_rate,
            "single_sample": f"{n_single} stamps, one initialiser + LM call per stamp, the reference's heuristic initial values",
            "learned_batched_over_plain_single": value / single_rate if single_rate else None,
            "learned_batched_over_plain_batched": value / (conv_p / (plain_ms * 1e-3)) if conv_p else None,
        },
        "clocks": clk.summary(),
        "e2e": {"value": converged_all / (e2e_ms * 1e-3), "unit": "fits/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "wall_ms_per_step": e2e_wall_ms,
                "path": "cnn.learned_fit_host: pinned host batches, the next batch uploaded on a copy stream "
                        "while the current one is fitted"},
        "roofline": roof,
        "roofline_integrate": roof_int,
        "autotune": tuned,
        "kernel_ms_per_step": {k: v[0] / args.steps for k, v in ktimes.items()},
        "kernel_launches_per_step": {k: v[1] / args.steps for k, v in ktimes.items()},
        "gpu_launches": launches,
        "work_per_step": {k: v / args.steps for k, v in work.items()},
    }

    if rank == 0 and not args.no_crowded:
        line["crowded_field"] = crowded_block(args, dev)
    if rank == 0 and not args.no_cnn:
        line["learned_init_cnn"] = cnn_block(args, dev)
    if rank == 0 and not args.no_configs:
        line["single_stamp_c0"] = c0_block(args, dev)
        line["batched_cutouts"] = cutouts_block(args, dev)
        line["bulge_disk_field"] = bulge_disk_block(args, dev)
    if rank == 0 and world == 1 and not args.no_cpu and args.cpu_sample > 0:
        from astrophot_gb300.transforms import rep_to_slots

        dh = data_h.numpy()
        sg = sigma_h.numpy()
        init_lh = init_l.cpu().numpy()
        vals_h = rep_to_slots(state.cpu().numpy(), init_lh, FREE_MASK)
        # stratified by signal-to-noise: the stamps sorted by peak (data - sky) / sigma, evenly
        # spaced; then up to 32 of the fits that did not end with "success"
        peak = (dh.reshape(S, -1) - 1.0).max(axis=1) / sg
        order = np.argsort(peak, kind="stable")
        k = min(args.cpu_sample, S)
        idx = [int(order[j]) for j in np.linspace(0, S - 1, k).round().astype(int)]
        chosen = set(idx)
        other = [int(i) for i in np.flatnonzero(status_h != N.LM_SUCCESS) if int(i) not in chosen][:32]

        def data_of(i):
            return dh[i * 4096 : (i + 1) * 4096].astype(np.float64).reshape(64, 64), float(sg[i])

        procs = max(1, min(os.cpu_count() or 1, k))
        for name, sel in (("parity", idx), ("parity_not_success", other)):
            if not sel:
                continue
            jobs = learned_sample_jobs(S, seed, sel, data_of=data_of, init_of=lambda i: init_lh[i])
            par, cpu = oracle_parity(jobs, [chi2_h[i] for i in sel], [vals_h[i] for i in sel],
                                     [N.LM_MESSAGES[int(status_h[i])] for i in sel], procs)
            line[name] = par
            if name == "parity":
                cpu["sample"] = (f"{k} stamps of this workload stratified by peak signal-to-noise, from the same "
                                 f"learned initial values; float64 numpy restatement of the reference LM on {procs} "
                                 "host processes")
                line["cpu_baseline"] = cpu
        par = line["parity"]
        # value counts converged fits (status); the sample's share within 1e-4 of the oracle's
        # chi^2 scales it (and e2e) when below 1
        share = par["within_1e-4"] / par["stamps"]
        line["value_within_1e-4_share"] = share
        line["value"] = value * share
        line["e2e"]["value"] = line["e2e"]["value"] * share
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


# ----------------------------------------------------------------------------------------
# crowded field: many galaxies on one image, joint LM (Group_Model + LM)
# ----------------------------------------------------------------------------------------


C0_KNOBS = {"sampling_mode": "midpoint_center", "integrate_mode": "none"}

def measured_peaks():
    """HBM copy bandwidth and dense bf16 throughput measured on this GPU model (the JSON file
    beside this script), else an earlier GB300 measurement (6.8 TB/s, 1.9 PFLOP/s)."""
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            z = json.load(f)
        return {"hbm_gbs": float(z["hbm_gbs"]), "bf16_tflops": float(z["bf16_tflops"]), "source": "measured"}
    except (OSError, KeyError, ValueError):
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


# algorithmic work of one stamp through the CNN: 2 * rows * K * N per layer, K the true
# reduction (9 taps of layer 1, not its zero padding to 16), N the true outputs (8 of layer 6)
CNN_FLOP_PER_STAMP = 2 * (1024 * 9 * 32 + 256 * 288 * 64 + 64 * 576 * 128 + 16 * 1152 * 256 + 4096 * 192 + 192 * 8)
# the least HBM traffic of an inference pass per stamp: the fp32 input stamp, the layer-1 im2col
# matrix (written, read), each bf16 activation written once and read once, the fp32 output row
CNN_BYTES_PER_STAMP = (4096 * 4 + 2 * 1024 * 16 * 2 + 2 * (1024 * 32 + 256 * 64 + 64 * 128 + 16 * 256 + 192) * 2
                       + 16 * 4)


def cnn_block(args, dev):
    """The learned initial guess's network on its own: inference over one 8,192-stamp chunk
    (the proposal's chunk) and Adam training steps (batch 512, the training batch, and 4,096),
    on the tcgen05 path and on the mma.sync path; then stamps/s of the whole training loop
    (rendering the training stamps included) on the tcgen05 path."""
    import ctypes

    import torch

    from astrophot_gb300 import _native as N
    from astrophot_gb300 import cnn

    peaks = measured_peaks()
    n = 8192
    net = cnn.InitNet(device=dev, seed=1)
    st = cnn.make_stamps(n, args.seed + 17, device=dev)
    x, lscale = net.prepare(st.data, st.sigma, n)
    raw = cnn._targets(torch.tensor(st.truth, device=dev), lscale)
    net.set_statistics(raw)
    t = ((raw - net.mean.double()) / net.std.double()).float().contiguous()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    lib = N.lib()
    old = cnn.get_tensor_path()
    out = {"chunk_stamps": n, "flop_per_stamp": CNN_FLOP_PER_STAMP, "min_bytes_per_stamp": CNN_BYTES_PER_STAMP,
           "peaks": peaks}
    try:
        for path in ("tcgen05", "mma_sync"):
            cnn.set_tensor_path(path)
            res = {}
            for _ in range(3):
                net.infer(x, n)
            torch.cuda.synchronize()
            reps = 10
            e0.record()
            for _ in range(reps):
                net.infer(x, n)
            e1.record()
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / reps
            tf = CNN_FLOP_PER_STAMP * n / (ms * 1e-3) / 1e12
            gbs = CNN_BYTES_PER_STAMP * n / (ms * 1e-3) / 1e9
            res["infer_ms_per_chunk"] = ms
            res["infer_stamps_per_s"] = n / (ms * 1e-3)
            res["infer_tflops"] = tf
            res["infer_frac_of_bf16_peak"] = tf / peaks["bf16_tflops"] if peaks.get("bf16_tflops") else None
            res["infer_min_traffic_gbs"] = gbs
            res["infer_frac_of_hbm_peak"] = gbs / peaks["hbm_gbs"] if peaks.get("hbm_gbs") else None
            for batch in (512, 4096):
                p0 = net.params.clone()
                m1 = torch.zeros_like(net.params)
                m2 = torch.zeros_like(net.params)
                grads = torch.zeros_like(net.params)
                loss = torch.zeros(1, dtype=torch.float64, device=dev)
                ws = net._workspace(batch)
                steps = n // batch

                def run(k0):
                    for j in range(steps):
                        b0 = j * batch
                        N.check(lib.ap_cnn_train_step(
                            N._ptr(net.params), N._ptr(net.params_bf16), N._ptr(grads), N._ptr(m1), N._ptr(m2),
                            N._ptr(x[b0 * 4096:]), N._ptr(t[b0:]), batch, ctypes.c_float(1e-4), k0 + j + 1,
                            ctypes.c_float(1e-4), N._ptr(loss), N._ptr(ws), ws.numel(), N._stream()),
                            "ap_cnn_train_step")

                run(0)
                torch.cuda.synchronize()
                e0.record()
                run(steps)
                e1.record()
                torch.cuda.synchronize()
                ms = e0.elapsed_time(e1)
                res[f"train_b{batch}_ms_per_step"] = ms / steps
                res[f"train_b{batch}_stamps_per_s"] = n / (ms * 1e-3)
                # forward + backward: three GEMMs of the forward's size per layer
                res[f"train_b{batch}_tflops"] = 3 * CNN_FLOP_PER_STAMP * n / (ms * 1e-3) / 1e12
                net.params.copy_(p0)
                net._sync_bf16()
            out[path] = res
        cnn.set_tensor_path("tcgen05")
        # whole training loop: stamps rendered on the GPU, prepared, then Adam steps of 512
        loop_stamps = 4 * n
        net2 = cnn.InitNet(device=dev, seed=2)
        net2.train(n_stamps=n, batch=512, chunk=n, seed=5)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        net2.train(n_stamps=loop_stamps, batch=512, chunk=n, seed=6)
        torch.cuda.synchronize()
        out["train_loop_stamps_per_s"] = loop_stamps / (time.perf_counter() - t0)
        out["train_loop"] = f"{loop_stamps} fresh rendered stamps, chunks of {n}, Adam batch 512, tcgen05 path"
        out["tc_status"] = cnn.tc_status()
    finally:
        cnn.set_tensor_path(old)
    out["tcgen05_over_mma_sync_infer"] = out["mma_sync"]["infer_ms_per_chunk"] / out["tcgen05"]["infer_ms_per_chunk"]
    out["tcgen05_over_mma_sync_train_b512"] = (out["mma_sync"]["train_b512_ms_per_step"]
                                              / out["tcgen05"]["train_b512_ms_per_step"])
    return out


def c0_block(args, dev):
    """The single-Sersic stamp configuration: 128 x 128 stamps of one Sersic galaxy + a locked sky
    of 1.0, a 25 x 25 Moffat PSF (FWHM 3 px, beta 3.5), midpoint sampling with 3 x 3
    Gauss-Legendre on the pixels within 2 px of the centre, noise sigma = sqrt(model + 10), LM
    of the 7 galaxy parameters from the truth perturbed by 10 %; ``--c0-stamps`` seeds fitted as
    one batch (fits/s), the oracle LM on a sample of them beside it (parity + CPU fits/s)."""
    import functools

    import torch

    from astrophot_gb300 import _native as N
    from astrophot_gb300 import synthetic
    from astrophot_gb300.transforms import rep_to_slots, slots_to_rep

    n = args.c0_stamps
    specs = [synthetic.c0_stamp(seed) for seed in range(n)]
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=FREE_MASK, has_sky=True, **C0_KNOBS)
    b = N.StampBatch([(128, 128)] * n, [(25, 25)] * n, N.scale_geometry(n), opts, dev)
    truth = np.array([np.r_[s.truth, 0.0] for s in specs])
    init = np.array([np.r_[s.init, 0.0] for s in specs])
    psf = b.pack_psf([s.psf for s in specs])
    models = b.unpack(b.render(torch.tensor(truth), psf))
    datas, ws = [], []
    for s_, m in zip(specs, models):
        d_, w_ = synthetic.add_noise(m.astype(np.float64), s_.seed)
        datas.append(d_)
        ws.append(w_)
    data, weight = b.pack(datas), b.pack(ws)
    fixed = torch.tensor(init, device=dev)
    rep0 = torch.tensor(slots_to_rep(init, FREE_MASK), device=dev)
    lmo = N.make_lm_options(rounds_per_sync=args.rounds_per_sync, use_graph=not args.no_graph)
    b.lm_fit(data, weight, None, psf, fixed, rep0, lmo)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3
    e0.record()
    for _ in range(reps):
        state, chi2, iters, status = b.lm_fit(data, weight, None, psf, fixed, rep0, lmo)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    st_h = status.cpu().numpy()
    conv = int(np.sum((st_h == N.LM_SUCCESS) | (st_h == N.LM_IMMOBILE)))
    out = {
        "workload": f"{n} stamps of 128x128, Sersic + locked sky 1.0, 25x25 Moffat (FWHM 3, beta 3.5), midpoint "
        "sampling + 3x3 Gauss-Legendre within 2 px of the centre, noise sqrt(model + 10), 7 parameters from "
        "the truth perturbed by 10 %, one batch",
        "fits_per_s": conv / (ms * 1e-3),
        "ms_per_batch": ms,
        "converged": conv,
        "mean_iterations": float(iters.cpu().numpy().mean()),
        "status_counts": {N.LM_MESSAGES[k]: int(np.sum(st_h == k)) for k in np.unique(st_h)},
    }
    if not args.no_cpu:
        k = min(args.c0_cpu_sample, n)
        idx = [int(i) for i in np.linspace(0, n - 1, k).round().astype(int)]
        dh, wh = data.cpu().numpy(), weight.cpu().numpy()
        vals = rep_to_slots(state.cpu().numpy(), init, FREE_MASK)
        c2 = chi2.cpu().numpy()
        jobs = [(dh[i * 16384 : (i + 1) * 16384].astype(np.float64).reshape(128, 128),
                 wh[i * 16384 : (i + 1) * 16384].astype(np.float64).reshape(128, 128),
                 specs[i].psf.astype(np.float32).astype(np.float64), init[i], truth[i]) for i in idx]
        procs = max(1, min(os.cpu_count() or 1, k))
        par, cpu = oracle_parity(jobs, [c2[i] for i in idx], [vals[i] for i in idx],
                                 [N.LM_MESSAGES[int(st_h[i])] for i in idx], procs,
                                 fit=functools.partial(_oracle_fit_full, knobs=C0_KNOBS))
        cpu["sample"] = f"{k} of the stamps, same data and initial values, {procs} host processes"
        out["parity"] = par
        out["cpu_baseline"] = cpu
    return out


def cutouts_block(args, dev):
    """The batched-cutout configuration: ``--cutout-stamps`` (8192) stamps with sides
    round(log-uniform(32, 256)) px, one Sersic + a locked sky of 1.0 each, its own Moffat PSF
    (FWHM U(2, 5) px, side odd(4 FWHM)), noise sqrt(model + 10), 7 parameters from the truth
    perturbed by 10 %, all fitted in one batched LM (persistent kernels, CUDA graphs, grid sizes
    from the in-project autotuner); the oracle LM on a size-stratified sample beside it."""
    import torch

    from astrophot_gb300 import _native as N
    from astrophot_gb300 import synthetic
    from astrophot_gb300.transforms import rep_to_slots, slots_to_rep

    specs = synthetic.cutout_stamps(args.cutout_stamps, args.seed + 17)
    S = len(specs)
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=FREE_MASK, has_sky=True)
    b = N.StampBatch([(s.nx, s.ny) for s in specs], [(s.psf.shape[1], s.psf.shape[0]) for s in specs],
                     N.scale_geometry(S), opts, dev)
    truth, init = truth_and_init_rows(specs)
    psf = b.pack_psf([s.psf for s in specs])
    models = b.unpack(b.render(torch.tensor(truth), psf))
    datas, ws = [], []
    for s_, m in zip(specs, models):
        d_, w_ = synthetic.add_noise(m.astype(np.float64), s_.seed)
        datas.append(d_)
        ws.append(w_)
    data, weight = b.pack(datas), b.pack(ws)
    fixed = torch.tensor(init, device=dev)
    rep0 = torch.tensor(slots_to_rep(init, FREE_MASK), device=dev)
    tuned = b.autotune(fixed, psf, jacobian=True)
    lmo = N.make_lm_options(rounds_per_sync=args.rounds_per_sync, use_graph=not args.no_graph)
    b.lm_fit(data, weight, None, psf, fixed, rep0, lmo)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 2
    e0.record()
    for _ in range(reps):
        state, chi2, iters, status = b.lm_fit(data, weight, None, psf, fixed, rep0, lmo)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    st_h = status.cpu().numpy()
    conv = int(np.sum((st_h == N.LM_SUCCESS) | (st_h == N.LM_IMMOBILE)))
    out = {
        "workload": f"{S} stamps, sides log-uniform 32-256 px ({int(b.out_pixels)} pixels), Sersic + locked sky "
        "1.0, own Moffat PSF FWHM U(2,5) side odd(4 FWHM), noise sqrt(model + 10), 7 parameters from the truth "
        "perturbed by 10 %, one batched LM",
        "fits_per_s": conv / (ms * 1e-3),
        "ms_per_batch": ms,
        "converged": conv,
        "mean_iterations": float(iters.cpu().numpy().mean()),
        "status_counts": {N.LM_MESSAGES[k]: int(np.sum(st_h == k)) for k in np.unique(st_h)},
        "autotune": tuned,
    }
    if not args.no_cpu:
        idx = sample_indices(specs, min(args.cutout_cpu_sample, S))
        dh, wh = data.cpu().numpy(), weight.cpu().numpy()
        vals = rep_to_slots(state.cpu().numpy(), init, FREE_MASK)
        c2 = chi2.cpu().numpy()
        jobs = []
        for i in idx:
            s_ = specs[i]
            o = b.out_offsets[i]
            jobs.append((dh[o : o + s_.nx * s_.ny].astype(np.float64).reshape(s_.ny, s_.nx),
                         wh[o : o + s_.nx * s_.ny].astype(np.float64).reshape(s_.ny, s_.nx),
                         s_.psf.astype(np.float32).astype(np.float64), init[i], truth[i]))
        procs = max(1, min(os.cpu_count() or 1, len(jobs)))
        par, cpu = oracle_parity(jobs, [c2[i] for i in idx], [vals[i] for i in idx],
                                 [N.LM_MESSAGES[int(st_h[i])] for i in idx], procs)
        cpu["sample"] = f"{len(idx)} stamps spread over the size range, same data and initial values, {procs} processes"
        out["parity"] = par
        out["cpu_baseline"] = cpu
    return out


def bulge_disk_block(args, dev):
    """The adjoint configuration at its stated size: 500 Sersic bulge (n ~ U(2, 6)) + exponential
    disk pairs sharing their centres (11 free parameters a pair, 5,500 in all) on a 2048 x 2048
    image with a 65 x 65 Moffat PSF (FWHM 3 px, beta 3.5; the configuration gives no FWHM), sky
    1.0, noise sqrt(model + 10), a window per pair.  Reports the render, the Jacobian + J^T W J,
    the adjoint of the chi^2 (VJP with the PSF-convolved tiles recomputed, not stored), the
    damped solve of the 5,500-parameter system and one LM iteration."""
    import torch

    from astrophot_gb300 import scene as SC
    from astrophot_gb300 import synthetic

    size = 2048
    truth, init, windows, psf = synthetic.bulge_disk_field(args.seed)
    zeros = np.zeros((size, size))
    sc_t = SC.Scene(size, size, synthetic.bulge_disk_sources(truth, windows), psf, zeros, zeros + 1, sky=1.0,
                    device=dev)
    model = sc_t.forward(sc_t.representation()).cpu().numpy().astype(np.float64).reshape(size, size)
    del sc_t
    data, weight = synthetic.add_noise(model, args.seed)
    sc = SC.Scene(size, size, synthetic.bulge_disk_sources(init, windows), psf, data, weight, sky=1.0, device=dev)
    rep = sc.representation()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 3

    def timed(fn):
        fn()
        fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            out = fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps, out

    fwd_ms, m = timed(lambda: sc.forward(rep))
    g = (sc.weight.double() * (m.double() - sc.data.double())).float()
    vjp_ms, _ = timed(lambda: sc.vjp(rep, g))

    def jac_hess():
        sc.jacobian(rep)
        return sc.hess()

    jac_ms, H = timed(jac_hess)
    grad = sc.jt(sc.residual(m))
    solve_ms, h_mixed = timed(lambda: sc.solve(H, grad, 1.0))
    solve64_ms, h64 = timed(lambda: sc.solve(H, grad, 1.0, mixed=False))
    solve_rel = float((h_mixed - h64).abs().max() / h64.abs().max())
    # untimed: first-call costs and the capture of each evaluation's graph (at its second call)
    SC.SceneLM(sc, initial_state=rep, max_iter=2).fit()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lm = SC.SceneLM(sc, initial_state=rep, max_iter=1).fit()
    torch.cuda.synchronize()
    lm_s = time.perf_counter() - t0
    return {
        "workload": f"{len(truth)} bulge (Sersic n U(2,6)) + exponential disk pairs sharing centres on {size}x{size}, "
        "65x65 Moffat (FWHM 3, beta 3.5), sky 1.0, noise sqrt(model + 10), a window per pair; "
        f"{sc.P} parameters (centre shared: 11 a pair)",
        "parameters": sc.P,
        "window_pairs": sc.n_pairs,
        "render_ms": fwd_ms,
        "render_mpix_per_s": size * size / (fwd_ms * 1e-3) / 1e6,
        "adjoint_vjp_ms": vjp_ms,
        "jacobian_and_jtwj_ms": jac_ms,
        "damped_solve_ms": solve_ms,
        "damped_solve_fp64_ms": solve64_ms,
        "damped_solve": "float32 Cholesky + float64 refinement (float64 factorisation when it does not converge); "
                        "max |h - h_fp64| / max |h_fp64| = %.1e" % solve_rel,
        "lm_iteration_s": lm_s,
        "chi2_ndf_start": float(lm.loss_history[0]),
        "chi2_ndf_after_one_iteration": float(lm.loss_history[-1]),
    }


def _oracle_source_window(job):
    """One Sersic source of a field rendered by the oracle on its own window with the group's
    working pixel count in its integration threshold (and its Jacobian when asked): (window
    model, seconds)."""
    params, window, psf, numel, grad, size = job
    from oracle.render import PSF, Component, Window, sample_component, sub_window

    cx, cy, q, PA, n, Re, Ie = params[:7]
    comp = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full",
                     psf_convolve_mode="direct", thr_numel=numel)
    win = sub_window(Window.from_scale(size, size), window)
    t = time.perf_counter()
    r = sample_component(comp, win, PSF(psf), grad=grad)
    return r.model, time.perf_counter() - t


def crowded_oracle(sc, rep, windows, psf, data, weight, sky, size, procs):
    """The crowded field's chi^2 / ndf at a joint vector from the oracle (every source on its own
    window, as the reference's pixels), and the oracle's CPU seconds for the render and for the
    Jacobians of all sources (one windowed LM iteration's model and Jacobian work)."""
    V = sc.values_matrix(rep)
    # the arrays the GPU fitted (float32)
    psf = psf.astype(np.float32).astype(np.float64)
    data = data.astype(np.float32).astype(np.float64)
    weight = weight.astype(np.float32).astype(np.float64)
    ky, kx = psf.shape
    numel = float((size + 2 * ((kx + 2) // 2)) * (size + 2 * ((ky + 2) // 2)))
    jobs = [(V[i], windows[i], psf, numel, False, size) for i in range(len(windows))]
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes=procs) as pool:
        res = pool.map(_oracle_source_window, jobs)
        k = min(len(jobs), 2 * procs)
        jres = pool.map(_oracle_source_window, [j[:4] + (True, size) for j in jobs[:k]])
    model = np.full((size, size), sky)
    for (m, _), w in zip(res, windows):
        (x0, x1), (y0, y1) = w
        model[y0:y1, x0:x1] += m
    chi2 = float(np.sum(weight * (data - model) ** 2) / max(1.0, size * size - sc.P))
    render_s = sum(t for _, t in res)
    jac_s = sum(t for _, t in jres) * len(jobs) / k
    return chi2, render_s, jac_s, k


def crowded_block(args, dev):
    """200 Sersic galaxies on a 1024 x 1024 image, 51 x 51 Gaussian PSF (sigma 2), sky 5.0,
    noise sigma = sqrt(model + 10), explicit per-galaxy windows; 1400 parameters fitted jointly
    for 20 LM iterations in the reference's default convolution mode "fft" (which takes FFT or
    direct convolution, whichever is faster for the kernel size).  Reports render Mpix/s,
    Jacobian build time and the LM run, and the render / Jacobian with every source convolved
    by FFT beside them."""
    import torch

    from astrophot_gb300 import scene as SC
    from astrophot_gb300 import synthetic

    size, n_src = args.crowded_size, args.crowded_sources
    truth, init, windows, psf = synthetic.crowded_field(args.seed, size, n_src)
    sky = 5.0
    src_t = [SC.SceneSource("sersic", list(t), w) for t, w in zip(truth, windows)]
    zeros = np.zeros((size, size))
    sc_t = SC.Scene(size, size, src_t, psf, zeros, zeros + 1, sky=sky, device=dev)
    model = sc_t.forward(sc_t.representation()).cpu().numpy().astype(np.float64).reshape(size, size)
    data, weight = synthetic.add_noise(model, args.seed)
    del sc_t
    src_i = [SC.SceneSource("sersic", list(t), w) for t, w in zip(init, windows)]
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    reps = 5

    def timed(sc, rep):
        for _ in range(2):
            sc.forward(rep)
            sc.jacobian(rep)
            sc.hess()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            sc.forward(rep)
        e1.record()
        torch.cuda.synchronize()
        fwd = e0.elapsed_time(e1) / reps
        e0.record()
        for _ in range(reps):
            sc.jacobian(rep)
            H = sc.hess()
        e1.record()
        torch.cuda.synchronize()
        return fwd, e0.elapsed_time(e1) / reps, H

    # every source convolved by FFT, for comparison
    sc_f = SC.Scene(size, size, src_i, psf, data, weight, sky=sky, device=dev,
                    options={"psf_convolve_mode": "fft", "fft_min_kernel": 1})
    rep = sc_f.representation()
    fwd_f, jac_f, _ = timed(sc_f, rep)
    chi2_f = float(sc_f.chi2(sc_f.forward(rep)))
    del sc_f
    # the reference's default mode "fft": FFT where it is faster for the kernel size, else direct
    sc = SC.Scene(size, size, src_i, psf, data, weight, sky=sky, device=dev, options={"psf_convolve_mode": "fft"})
    fwd_ms, jac_ms, H = timed(sc, rep)
    # a damping trial rendered as its difference to the recorded base render
    xd = torch.tensor(rep, device=dev)
    vd = torch.tensor(np.random.default_rng(args.seed).normal(size=sc.P) * 1e-3, device=dev)
    sc.set_stage_base(rep)
    sc.forward_base_device(xd)
    for _ in range(2):
        sc.forward_diff_device(xd, vd, 1.0)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        sc.forward_diff_device(xd, vd, 1.0)
    e1.record()
    torch.cuda.synchronize()
    diff_ms = e0.elapsed_time(e1) / reps
    chi2_d = float(sc.chi2(sc.forward(rep)))
    g = sc.jt(sc.residual(sc.forward(rep)))
    torch.cuda.synchronize()
    e0.record()
    for _ in range(reps):
        h_mixed = sc.solve(H, g, 1.0)
    e1.record()
    torch.cuda.synchronize()
    solve_ms = e0.elapsed_time(e1) / reps
    e0.record()
    for _ in range(reps):
        h64 = sc.solve(H, g, 1.0, mixed=False)
    e1.record()
    torch.cuda.synchronize()
    solve64_ms = e0.elapsed_time(e1) / reps
    solve_rel = float((h_mixed - h64).abs().max() / h64.abs().max())
    # two untimed LM iterations of each loop first (first-call costs of the process: device
    # allocations of the LM's vectors and images, first launches, and the capture of every
    # evaluation's CUDA graph, which happens at its second call), as the other blocks warm up
    SC.SceneLM(sc, initial_state=rep, max_iter=2).fit()
    SC.SceneLM(sc, initial_state=rep, max_iter=2, precise_trials=False).fit()
    SC.SceneLM(sc, initial_state=rep, max_iter=2, device_loop=False).fit()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    lm = SC.SceneLM(sc, initial_state=rep, max_iter=args.crowded_iters).fit()
    torch.cuda.synchronize()
    lm_s = time.perf_counter() - t0
    # the device loop with full float32 trial renders (no base render per step; the accepted
    # trial's render is the next base image) and the same LM driven from the host (host
    # staging, four reads per damping trial), which takes the same steps
    t0 = time.perf_counter()
    lm_p = SC.SceneLM(sc, initial_state=rep, max_iter=args.crowded_iters, precise_trials=False).fit()
    torch.cuda.synchronize()
    lm_plain_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    lm_h = SC.SceneLM(sc, initial_state=rep, max_iter=args.crowded_iters, device_loop=False).fit()
    torch.cuda.synchronize()
    lm_host_s = time.perf_counter() - t0
    # device time the LM's work takes at the kernel times measured above: a Jacobian + J^T W J
    # per iteration, a damped solve per trial, its render and the geodesic term's (full or as a
    # difference), the base renders (every difference step's, and those not taken from an
    # accepted trial)
    floor_ms = (lm.iterations * jac_ms + lm.trials * solve_ms + lm.full_renders * fwd_ms
                + lm.diff_renders * diff_ms + (1 + lm.base_renders) * fwd_ms)
    out = {
        "workload": f"{n_src} Sersic galaxies on a {size}x{size} image, 51x51 Gaussian PSF (sigma 2; mode fft: "
        "the convolution takes the faster of FFT and direct for the kernel size, direct at 53x53), sky 5.0, "
        "explicit windows (half-size 4 Re + 3 sigma + 2), noise sqrt(model + 10); "
        f"{sc.P} parameters fitted jointly",
        "parameters": sc.P,
        "window_pairs": sc.n_pairs,
        "render_ms": fwd_ms,
        "render_mpix_per_s": size * size / (fwd_ms * 1e-3) / 1e6,
        "difference_render_ms": diff_ms,
        "jacobian_build_ms": jac_ms,
        "all_fft_convolution": {"render_ms": fwd_f, "jacobian_build_ms": jac_f,
                                "chi2_rel_diff_vs_direct": abs(chi2_f / chi2_d - 1)},
        "damped_solve_ms": solve_ms,
        "damped_solve_fp64_ms": solve64_ms,
        "damped_solve": "float32 Cholesky + float64 refinement (float64 factorisation when it does not converge); "
                        "max |h - h_fp64| / max |h_fp64| = %.1e" % solve_rel,
        "lm_fp64_retries": lm.fp64_retries,
        "lm_iterations": lm.iterations,
        "lm_seconds": lm_s,
        "lm_ms_per_iteration": lm_s * 1e3 / max(lm.iterations, 1),
        "lm_damping_trials": lm.trials,
        "lm_difference_steps": lm.diff_steps,
        "lm_geodesic_trials": lm.geodesic_trials,
        "lm_kernel_floor_ms_per_iteration": floor_ms / max(lm.iterations, 1),
        "lm_loop": "device vectors, parameters staged on the device, one status read per damping trial; "
                   "once a step gains less than 1 %, trials and geodesic renders as differences to the "
                   "step's recorded base render",
        "lm_full_trials_ms_per_iteration": lm_plain_s * 1e3 / max(lm_p.iterations, 1),
        "lm_full_trials_iterations": lm_p.iterations,
        "lm_full_trials_message": lm_p.message,
        "lm_host_loop_ms_per_iteration": lm_host_s * 1e3 / max(lm_h.iterations, 1),
        "lm_host_loop_same_trajectory": bool(lm_h.message == lm_p.message and lm_h.iterations == lm_p.iterations
                                             and np.allclose(lm_h.loss_history, lm_p.loss_history, rtol=1e-9)),
        "chi2_ndf_start": lm.loss_history[0],
        "chi2_ndf_end": min(lm.loss_history),
        "lm_message": lm.message,
    }
    if not args.no_cpu:
        procs = os.cpu_count() or 1
        c2o, rs, js, k = crowded_oracle(sc, lm.res(), windows, psf, data, weight, sky, size, procs)
        out["oracle"] = {
            "chi2_ndf_at_fitted_state": c2o,
            "rel_diff_vs_gpu": abs(min(lm.loss_history) / c2o - 1.0),
            "cpu_render_s": rs,
            "cpu_jacobian_s": js,
            "cpu_iteration_s": rs + js,
            "sample": f"every source rendered by the float64 oracle on its own window (the group's working "
            f"pixel count in its threshold), {procs} processes; Jacobians timed on {k} sources and scaled to "
            f"{len(windows)}; one LM iteration's render + Jacobian work, CPU seconds summed over sources",
        }
    return out


def _oracle_init(data):
    """The reference's initialize() heuristics restated in float64 (oracle) on one stamp."""
    from oracle.refinit import initialize

    t = time.perf_counter()
    o = initialize(data, "sersic", 1.0)
    v = np.r_[o["center"], o["q"], o["PA"], o["n"], o["Re"], o["Ie"]]
    return v, time.perf_counter() - t


INIT_METRIC = "initial-value heuristics (the reference's initialize()) stamps/s"


def run_gpu_init(args):
    """--workload init: the reference's initialiser (``ap_reference_init``) on the learned
    workload's stamps; value = stamps/s with the stamps resident in HBM, e2e through host
    buffers; parity and the CPU baseline from the float64 oracle on --cpu-sample stamps."""
    import torch

    from astrophot_gb300 import cnn

    rank, world, local = rank_info()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    S = args.stamps
    st = cnn.make_stamps(S, args.seed + 7919 * rank, device=dev)
    data_h = st.data.cpu().pin_memory()
    for _ in range(max(args.warmup, 0)):
        cnn.heuristic_init(st, S)
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            vals = cnn.heuristic_init(st, S)
        e1.record()
        torch.cuda.synchronize()
    dev_ms = e0.elapsed_time(e1) / args.steps

    def step_e2e():
        ss = cnn.StampSet(st.truth, data_h.to(dev, non_blocking=True), st.weight, st.psf, st.sigma, st.batch)
        return cnn.heuristic_init(ss, S).cpu()

    step_e2e()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        step_e2e()
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    dev_ms, e2e_ms, _, total = aggregate_ranks(dev_ms, e2e_ms, S, S, dev)
    if rank != 0:
        return
    line = {
        "metric": INIT_METRIC,
        "value": total / (dev_ms * 1e-3),
        "unit": "stamps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": f"reference initialiser on {S} held-out 64x64 stamps of the learned workload per GPU",
                   "stamps_per_gpu": S, "l2": "the stamps (1 GB at 65536) exceed the 129 MB L2"},
        "clocks": clk.summary(),
        "e2e": {"value": total / (e2e_ms * 1e-3), "unit": "stamps/s", "h2d_bytes_per_step": int(data_h.numel() * 4),
                "d2h_bytes_per_step": int(S * 8 * 8)},
        "gpu_launches": args.steps,
    }
    if not args.no_cpu:
        k = min(args.cpu_sample, S)
        idx = np.linspace(0, S - 1, k).round().astype(int)
        data = st.data.view(S, 64, 64)[torch.as_tensor(idx, device=dev)].cpu().numpy().astype(np.float64)
        got = vals.cpu().numpy()[idx, :7]
        res = [_oracle_init(d) for d in data]
        ref = np.array([r[0] for r in res])
        secs = sum(r[1] for r in res)
        err = np.abs(got - ref) / np.maximum(1.0, np.abs(ref))
        line["cpu_baseline"] = {"value": k / secs, "unit": "stamps/s", "cores": 1, "kind": "port",
                                "sample": f"{k} stamps, float64 numpy restatement of the reference initialize(), one core"}
        line["parity"] = {"stamps": int(k), "q_equal": int(np.sum(got[:, 2] == ref[:, 2])),
                          "max_rel_err_centre_pa": float(err[:, [0, 1, 3]].max()),
                          "max_rel_err_n_re_ie": float(err[:, 4:].max())}
    print(json.dumps(line), flush=True)


def run_reference_init(args):
    """--impl reference --workload init: the float64 restatement of the reference's initialize()
    over all host cores on a bounded sample of the same stamps."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    from astrophot_gb300 import cnn  # noqa: F401  (stamp draws only; no GPU work)

    cores = os.cpu_count() or 1
    k = min(args.stamps, 4 * cores)
    idx = list(np.linspace(0, args.stamps - 1, k).round().astype(int))
    jobs = learned_sample_jobs(args.stamps, args.seed, idx)
    datas = [j[0] for j in jobs]
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes=min(cores, len(datas))) as pool:
        if args.warmup > 0:
            pool.map(_oracle_init, datas[: min(len(datas), cores)])
        times = []
        for _ in range(args.steps):
            t = time.perf_counter()
            pool.map(_oracle_init, datas)
            times.append(time.perf_counter() - t)
    dt = statistics.median(times)
    value = len(datas) / dt
    line = {
        "impl": "reference", "metric": INIT_METRIC, "value": value, "unit": "stamps/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"reference initialiser on {args.stamps} held-out 64x64 stamps of the learned workload",
                   "sample": f"{len(datas)} stamps evenly spaced over the workload, {min(cores, len(datas))} processes"},
        "cpu_baseline": {"value": value, "unit": "stamps/s", "cores": min(cores, len(datas)), "kind": "port",
                         "sample": f"{len(datas)} stamps (float64 numpy restatement of the reference initialize())"},
        "e2e": {"value": value, "unit": "stamps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ----------------------------------------------------------------------------------------
# fitted PSF models
# ----------------------------------------------------------------------------------------
LIVEPSF_METRIC = "LM fits/s of galaxy + live Moffat PSF model (9 parameters, chi2 within 1e-4 of the FP64 oracle)"
LIVEPSF_SIZE, LIVEPSF_K = 64, 15


def livepsf_specs(n, seed):
    """Truth and initial values of ``n`` stamps: (psf {n, Rd}, galaxy [cx, cy, q, PA, n, Re, Ie])."""
    rng = np.random.default_rng(seed + 104729)
    out = []
    c = LIVEPSF_SIZE / 2
    for i in range(n):
        tp = dict(n=float(rng.uniform(2.0, 4.0)), Rd=float(rng.uniform(1.5, 2.8)))
        tg = [c + rng.uniform(-1, 1), c + rng.uniform(-1, 1), rng.uniform(0.5, 0.85), rng.uniform(0.2, 2.9),
              rng.uniform(1.0, 3.0), rng.uniform(1.2, 2.5), rng.uniform(2.0, 2.8)]
        ip = dict(n=tp["n"] * 0.85, Rd=tp["Rd"] * 1.15)
        ig = [tg[0] + 0.3, tg[1] - 0.3, min(tg[2] * 1.08, 0.95), tg[3] + 0.1, tg[4] * 1.15, tg[5] * 1.15, tg[6] - 0.1]
        out.append(dict(truth=dict(psf=tp, gal=[float(v) for v in tg]), init=dict(psf=ip, gal=[float(v) for v in ig]),
                        seed=seed + 31 * i))
    return out


def _oracle_livepsf(job):
    """(final chi2/ndf, final vector, seconds) of the float64 oracle LM on one stamp."""
    from oracle.lm import LMOracle
    from oracle.psfmodel import LivePSFProblem
    from oracle.render import Component, Window

    data, weight, init = job
    cx, cy, q, PA, n, Re, Ie = init["gal"]
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
    t = time.perf_counter()
    pr = LivePSFProblem(gal, Window.from_scale(LIVEPSF_SIZE, LIVEPSF_SIZE), dict(init["psf"], I0=0.0),
                        (LIVEPSF_K, LIVEPSF_K), data, weight)
    lm = LMOracle(pr)
    lm.fit()
    return float(np.min(lm.loss_history)), pr.values(), time.perf_counter() - t


def _oracle_livepsf_truth(spec):
    """Noisy data of one stamp rendered by the float64 restatement (the reference arm's input)."""
    from oracle.psfmodel import LivePSFProblem
    from oracle.render import Component, Window

    from astrophot_gb300 import synthetic

    cx, cy, q, PA, n, Re, Ie = spec["truth"]["gal"]
    gal = Component("sersic", {"center": [cx, cy], "q": q, "PA": PA, "n": n, "Re": Re, "Ie": Ie}, psf_mode="full")
    z = np.zeros((LIVEPSF_SIZE, LIVEPSF_SIZE))
    pr = LivePSFProblem(gal, Window.from_scale(LIVEPSF_SIZE, LIVEPSF_SIZE), dict(spec["truth"]["psf"], I0=0.0),
                        (LIVEPSF_K, LIVEPSF_K), z, z + 1)
    img = pr.forward(pr.representation()).reshape(LIVEPSF_SIZE, LIVEPSF_SIZE)
    return synthetic.add_noise(img, spec["seed"])


def crowded_live_psf_block(args, dev):
    """200 Sersic galaxies on 1024 x 1024 convolved with one live 31 x 31 Moffat PSF model whose n
    and Rd are fitted with them (1402 parameters): Jacobian build (with the two image-wide PSF
    columns) and the scene LM."""
    import torch

    from astrophot_gb300 import scene as SC
    from astrophot_gb300 import synthetic

    size, n_src = args.crowded_size, args.crowded_sources
    truth, init, windows, _ = synthetic.crowded_field(args.seed, size, n_src)
    sky = 5.0
    tp, ip = dict(n=3.0, Rd=2.5, I0=0.0), dict(n=2.6, Rd=2.8, I0=0.0)
    zeros = np.zeros((size, size))
    sc_t = SC.Scene(size, size, [SC.SceneSource("sersic", list(t), w) for t, w in zip(truth, windows)], None, zeros,
                    zeros + 1, sky=sky, device=dev, psf_model=SC.LivePSF(tp, (31, 31), device=dev))
    model = sc_t.forward(sc_t.representation()).cpu().numpy().astype(np.float64).reshape(size, size)
    data, weight = synthetic.add_noise(model, args.seed)
    del sc_t
    sc = SC.Scene(size, size, [SC.SceneSource("sersic", list(t), w) for t, w in zip(init, windows)], None, data,
                  weight, sky=sky, device=dev, options={"psf_convolve_mode": "fft"},
                  psf_model=SC.LivePSF(ip, (31, 31), device=dev))
    rep = sc.representation()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for _ in range(2):
        sc.forward(rep)
        sc.jacobian(rep)
        sc.hess()
    torch.cuda.synchronize()
    reps = 5
    e0.record()
    for _ in range(reps):
        sc.forward(rep)
    e1.record()
    torch.cuda.synchronize()
    fwd_ms = e0.elapsed_time(e1) / reps
    e0.record()
    for _ in range(reps):
        sc.jacobian(rep)
        sc.hess()
    e1.record()
    torch.cuda.synchronize()
    jac_ms = e0.elapsed_time(e1) / reps
    t0 = time.perf_counter()
    lm = SC.SceneLM(sc, initial_state=rep, max_iter=args.crowded_iters).fit()
    torch.cuda.synchronize()
    lm_s = time.perf_counter() - t0
    return {
        "workload": f"{n_src} Sersic galaxies on a {size}x{size} image sharing one live 31x31 Moffat PSF model "
        f"(truth n 3.0, Rd 2.5; start 2.6, 2.8), sky 5.0, explicit windows; {sc.P} parameters fitted jointly",
        "parameters": sc.P,
        "render_ms": fwd_ms,
        "jacobian_and_hessian_ms": jac_ms,
        "lm_iterations": lm.iterations,
        "lm_seconds": lm_s,
        "lm_ms_per_iteration": lm_s * 1e3 / max(lm.iterations, 1),
        "chi2_ndf_start": lm.loss_history[0],
        "chi2_ndf_end": min(lm.loss_history),
        "psf_fitted": {"n": sc.live_psf.params["n"], "Rd": sc.live_psf.params["Rd"], "truth_n": 3.0, "truth_Rd": 2.5},
        "lm_message": lm.message,
    }


def run_gpu_livepsf(args):
    """--workload livepsf: fits/s of galaxy + live PSF stamps, each fitted by the scene LM
    (device-resident data: value; host data copied in and the fitted vector read back: e2e)."""
    import torch

    from astrophot_gb300 import scene as SC
    from astrophot_gb300 import synthetic

    rank, world, local = rank_info()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    dev = torch.device("cuda", torch.cuda.current_device())
    S = args.stamps
    specs = livepsf_specs(S, args.seed + 7919 * rank)
    z = np.zeros((LIVEPSF_SIZE, LIVEPSF_SIZE))
    scenes, inits, hosts = [], [], []
    for sp in specs:
        sc_t = SC.Scene(LIVEPSF_SIZE, LIVEPSF_SIZE, [SC.SceneSource("sersic", sp["truth"]["gal"])], None, z, z + 1,
                        device=dev, psf_model=SC.LivePSF(dict(sp["truth"]["psf"], I0=0.0), (LIVEPSF_K, LIVEPSF_K),
                                                         device=dev))
        img = sc_t.forward(sc_t.representation()).cpu().numpy().astype(np.float64).reshape(LIVEPSF_SIZE, LIVEPSF_SIZE)
        data, weight = synthetic.add_noise(img, sp["seed"])
        sc = SC.Scene(LIVEPSF_SIZE, LIVEPSF_SIZE, [SC.SceneSource("sersic", sp["init"]["gal"])], None, data, weight,
                      device=dev, psf_model=SC.LivePSF(dict(sp["init"]["psf"], I0=0.0), (LIVEPSF_K, LIVEPSF_K),
                                                       device=dev))
        scenes.append(sc)
        inits.append(sc.representation())
        hosts.append(torch.from_numpy(data.astype(np.float32).reshape(-1)).pin_memory())

    def step(e2e=False, concurrent=False):
        if e2e:
            for sc, h in zip(scenes, hosts):
                sc.data.copy_(h, non_blocking=True)
        if concurrent:
            lms = SC.fit_scenes(scenes, inits, workers=args.livepsf_workers)
        else:
            lms = [SC.SceneLM(sc, initial_state=x0.copy()).fit() for sc, x0 in zip(scenes, inits)]
        return [(min(lm.loss_history), lm.res(), lm.message) for lm in lms]

    for _ in range(max(args.warmup, 0)):
        res = step()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record()
        for _ in range(args.steps):
            res = step()
        e1.record()
        torch.cuda.synchronize()
    dev_ms = e0.elapsed_time(e1) / args.steps
    e0.record()
    for _ in range(args.steps):
        step(e2e=True)
    e1.record()
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    e0.record()
    con = step(concurrent=True)
    e1.record()
    torch.cuda.synchronize()
    con_ms = e0.elapsed_time(e1)
    same = all(a[2] == b[2] and a[0] == b[0] for a, b in zip(res, con))
    converged = sum(1 for r in res if r[2].startswith("success"))
    dev_ms, e2e_ms, converged, total = aggregate_ranks(dev_ms, e2e_ms, converged, S, dev)
    if rank != 0:
        return
    line = {
        "metric": LIVEPSF_METRIC,
        "value": converged / (dev_ms * 1e-3),
        "unit": "fits/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": dev_ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 render / f64 LM",
        "data": "synthetic",
        "config": {"workload": f"{S} stamps of {LIVEPSF_SIZE}x{LIVEPSF_SIZE} per GPU, compact Sersic (Re 1.2-2.5 px) "
                   f"convolved with a live Moffat PSF model on {LIVEPSF_K}x{LIVEPSF_K} (truth n 2-4, Rd 1.5-2.8), "
                   "noise sqrt(model + 10); PSF n, Rd + 7 galaxy parameters fitted by the scene LM, one stamp after "
                   "another",
                   "stamps_per_gpu": S,
                   "l2": "small stamps: resident in L2 (a host-driven LM per stamp, latency-bound)"},
        "fits": {"total": total, "converged": converged,
                 "messages": {m: sum(1 for r in res if r[2] == m) for m in sorted({r[2] for r in res})}},
        "concurrent": {"fits_per_s": S / (con_ms * 1e-3), "ms_per_step": con_ms,
                       "fits_at_a_time": min(args.livepsf_workers, S), "same_fits": bool(same),
                       "note": "host threads with one CUDA stream each (fit_scenes): the per-fit host work holds "
                               "the GIL, so overlapping fits does not raise throughput"},
        "clocks": clk.summary(),
        "e2e": {"value": converged / (e2e_ms * 1e-3), "unit": "fits/s",
                "h2d_bytes_per_step": int(S * LIVEPSF_SIZE * LIVEPSF_SIZE * 4), "d2h_bytes_per_step": int(S * 9 * 8)},
        "roofline": None,
        "roofline_note": "each LM iteration launches ~100 small kernels on a 64x64 stamp and reads the damped step "
                         "status and chi2 back to the host: bound by launch latency and host round trips, not by a "
                         "unit; concurrent fits overlap them",
    }
    if not args.no_crowded:
        line["crowded_live_psf"] = crowded_live_psf_block(args, dev)
    if not args.no_cpu:
        k = min(args.cpu_sample, S)
        idx = list(np.linspace(0, S - 1, k).round().astype(int))
        jobs = [(scenes[i].data.cpu().numpy().astype(np.float64).reshape(LIVEPSF_SIZE, LIVEPSF_SIZE),
                 scenes[i].weight.cpu().numpy().astype(np.float64).reshape(LIVEPSF_SIZE, LIVEPSF_SIZE),
                 specs[i]["init"]) for i in idx]
        out = [_oracle_livepsf(j) for j in jobs]
        secs = sum(o[2] for o in out)
        rel = [abs(res[i][0] / o[0] - 1) for i, o in zip(idx, out)]
        line["cpu_baseline"] = {"value": k / secs, "unit": "fits/s", "cores": 1, "kind": "port",
                                "sample": f"{k} stamps of this workload, float64 numpy restatement of the reference "
                                          "(live PSF sampling + LM), one core"}
        line["parity"] = {"stamps": k, "max_rel_chi2_vs_oracle": float(max(rel)),
                          "within_1e-4": int(sum(r <= 1e-4 for r in rel))}
    print(json.dumps(line), flush=True)


def run_reference_livepsf(args):
    """--impl reference --workload livepsf: the float64 restatement (live PSF sampling + LM) on
    all host cores, on the same stamps (rendered and noised by the restatement)."""
    rank, world, _ = rank_info()
    if rank != 0:
        return
    cores = os.cpu_count() or 1
    specs = livepsf_specs(args.stamps, args.seed)
    k = min(args.stamps, 2 * cores)
    specs = [specs[i] for i in np.linspace(0, args.stamps - 1, k).round().astype(int)]
    ctx = mp.get_context("spawn")
    with ctx.Pool(processes=min(cores, len(specs))) as pool:
        dw = pool.map(_oracle_livepsf_truth, specs)
        jobs = [(d, w, sp["init"]) for (d, w), sp in zip(dw, specs)]
        if args.warmup > 0:
            pool.map(_oracle_livepsf, jobs[: min(len(jobs), cores)])
        times = []
        for _ in range(args.steps):
            t = time.perf_counter()
            pool.map(_oracle_livepsf, jobs)
            times.append(time.perf_counter() - t)
    dt = statistics.median(times)
    value = len(jobs) / dt
    line = {
        "impl": "reference", "metric": LIVEPSF_METRIC, "value": value, "unit": "fits/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.stamps} stamps of {LIVEPSF_SIZE}x{LIVEPSF_SIZE}, Sersic + live Moffat PSF model "
                               f"on {LIVEPSF_K}x{LIVEPSF_K}, 9 parameters fitted",
                   "sample": f"{len(jobs)} stamps evenly spaced over the workload, {min(cores, len(jobs))} processes"},
        "cpu_baseline": {"value": value, "unit": "fits/s", "cores": min(cores, len(jobs)), "kind": "port",
                         "sample": f"{len(jobs)} stamps (float64 numpy restatement of live PSF sampling + LM)"},
        "e2e": {"value": value, "unit": "fits/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.cpu_sample is None:
        args.cpu_sample = 256 if args.workload in ("learned", "cutouts") else 8
    if args.impl == "reference":
        if args.workload == "learned":
            run_reference_learned(args)
        elif args.workload == "init":
            run_reference_init(args)
        elif args.workload == "livepsf":
            run_reference_livepsf(args)
        elif args.workload == "crowded":
            print(json.dumps({"impl": "reference", "workload": "crowded",
                              "unavailable": "the crowded-field block is a GPU-only secondary measurement"}))
        else:
            run_reference(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
