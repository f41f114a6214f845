#!/usr/bin/env python
"""Throughput of the ensemble stretch-move engine: walker-steps/s on the 50-dimensional
correlated Gaussian workload (AR(1) covariance, rho = 0.9, per-dimension scales
log-uniform in [0.1, 10], precision matrix as 2500 hyperparameters; 65,536 walkers
initialised N(0, I); 2,000 burn-in and 4,000 sampling steps; outputs mean, variance,
acor and 128-bin histograms).

One step = that whole job on one GPU.  `value` times it with the inputs resident on the
device; `e2e` times the same job through the C ABI from host buffers (sampler creation
with the host copy of the precision matrix, results copied back).  The reference arm
(--impl reference) times the CPU restatement of the reference's stretch kernel on the
host cores.  Multi-GPU: independent replicas (the path has no exchange step).
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402

DIM = 50
WALKERS = 65536
BURN = 2000
RUN = 4000
BINS = 128
SEED = 0
BYTES_PER_WALKER_STEP = 12 * DIM + 8      # read self + partner, write on accept, 2 logfn
FLOP_PER_WALKER_STEP = 2 * DIM * DIM      # dense -x'Px/2
L2_FLUSH_BYTES = 256 << 20


def precision_matrix(dim=DIM, seed=SEED):
    """Sigma_ij = s_i s_j rho^|i-j|, rho = 0.9, s_i log-uniform in [0.1, 10]; returns
    (P = Sigma^-1 as float32, Sigma as float64)."""
    rng = np.random.default_rng(seed)
    s = np.exp(rng.uniform(np.log(0.1), np.log(10.0), dim))
    i = np.arange(dim)
    sigma = np.outer(s, s) * 0.9 ** np.abs(i[:, None] - i[None, :])
    return np.linalg.inv(sigma).astype(np.float32), sigma


class ClockSampler:
    """nvidia-smi SM clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return j.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = os.path.join(ROOT, "profiles", "stretch_tcr_mvn50.txt")
    if not os.path.exists(p):
        return None
    for ln in open(p):
        if ln.startswith("traffic_bytes_per_launch_full_size:"):
            try:
                return float(ln.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


# ------------------------------------------------------------------ CPU (oracle) timing
def cpu_sample(steps_budget_s=12.0, walkers=WALKERS):
    """The CPU restatement of the reference's stretch kernel (OpenMP over walkers, all
    host cores) on the same workload: bounded to about steps_budget_s of CPU work."""
    from oracle import oracle as O
    P, _ = precision_matrix()
    threads = os.cpu_count() or 1
    r = O.Stretch("mvn_precision", DIM, walkers, P.reshape(-1), seed=SEED, threads=threads,
                  flags=O.ACCEPT_LOG64)
    r.init_position_normal(SEED + 1)
    t0 = time.perf_counter()
    r.move_bare()
    t1 = time.perf_counter() - t0
    n = max(1, int(steps_budget_s / max(t1, 1e-6)))
    t0 = time.perf_counter()
    for _ in range(n):
        r.move_bare()
    dt = time.perf_counter() - t0
    return {"value": walkers * n / dt, "unit": "walker-steps/s", "cores": threads, "kind": "port",
            "sample": "%d ensemble steps of the %d-walker 50-D job (%.1f s)" % (n, walkers, dt)}


def max_over_ranks(t, dist, device):
    """The timed region's length, maximised over the ranks: the slowest replica bounds the
    whole job.  One rank (dist None) returns t unchanged."""
    if dist is None:
        return float(t)
    import torch
    x = torch.tensor([float(t)], dtype=torch.float64, device=device)
    dist.all_reduce(x, op=dist.ReduceOp.MAX)
    return float(x.item())


def replica_throughput(jobs, world, t_total):
    """Whole-job walker-steps/s of `world` replicas that each ran `jobs` full jobs."""
    return WALKERS * (BURN + RUN) * jobs * world / t_total


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    budget = max(3.0, min(20.0, 60.0 / max(1, args.steps + args.warmup)))
    for _ in range(args.warmup):
        cpu_sample(budget / 4)
    vals = [cpu_sample(budget) for _ in range(args.steps)]
    v = statistics.median(x["value"] for x in vals)
    line = {
        "impl": "reference", "metric": "walker-steps/s", "value": v, "unit": "walker-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * WALKERS * (BURN + RUN) / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": config(),
        "cpu_baseline": {"value": v, "unit": "walker-steps/s", "cores": vals[0]["cores"],
                         "kind": "port", "sample": vals[0]["sample"]},
        "e2e": {"value": v, "unit": "walker-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def config():
    return {"workload": "mvn50-ar1 (50-D correlated Gaussian, rho 0.9, scales log-U[0.1,10])",
            "dim": DIM, "walkers": WALKERS, "burn_in": BURN, "run": RUN, "bins": BINS,
            "model_form": "gemm on the tensor cores (64-walker tiles, x'Px as a tcgen05 "
                          "split-bf16 product, fp32 accumulation, resident precision matrix)",
            "l2": "flushed between timed steps (256 MiB device write)",
            "parallelism": "replicas"}


# ------------------------------------------------------------------ other workloads
# (measured with --config; the default line above is the 50-D Gaussian job)
def _workload(name, rows=0):
    """(model factory args, params builder, walkers, burn, run, bins, init, algorithmic
    FLOP and bytes per walker-step, description) of the other benchmark workloads."""
    import torch
    from bayadera_gb300 import models as M
    if name == "c1":
        rng = np.random.default_rng(0)
        data = rng.normal(3.0, 2.0, 10000).astype(np.float32)
        params = np.concatenate([data, np.array([0.0, 10.0, 0.0, 20.0], np.float32)])
        return dict(model=M.gaussian_posterior_model(), fast="tiled", params=params,
                    walkers=4096, burn=512, run=1024, bins=256,
                    init=lambda s, seed: s.init_position(seed, [2.0, 4.0, 1.0, 3.0]),
                    flop=3 * 10000, bytes=0,
                    desc="2-D Gaussian (mu, sigma) posterior, N=10,000 data, prior "
                         "N(0,10^2) x U(0,20)")
    if name == "c3":
        n, F = rows or (1 << 20), 64
        rng = np.random.default_rng(0)
        X = rng.standard_normal((n, F), dtype=np.float32)
        beta = rng.normal(0.0, 1.0 / 8.0, F)
        eta = X.astype(np.float64) @ beta
        y = (rng.random(n) < 1.0 / (1.0 + np.exp(-eta))).astype(np.float32)
        rows = np.empty((n, F + 1), np.float32)
        rows[:, :F] = X
        rows[:, F] = y
        params = torch.from_numpy(np.concatenate([rows.reshape(-1), [5.0]]).astype(np.float32)).cuda()
        return dict(model=M.logistic_model(F), fast="tensor", forms=("tensor", "gemm", "plain"),
                    params=params, walkers=8192,
                    burn=10, run=20, bins=128, plain_burn=1, plain_run=4, rows=n,
                    row_len=F + 1, hyper_len=1,
                    init=lambda s, seed: s.init_position_normal(seed, 0.0, 0.05),
                    flop=2 * F * n, bytes=4 * (F + 1) * n // (8192 // 2),
                    desc="Bayesian logistic regression, X 1,048,576 x 64 N(0,1), beta* ~ "
                         "N(0,1/64), prior N(0,5^2 I)")
    if name == "c5":
        n, F = rows or (1 << 24), 256
        rng = np.random.default_rng(0)
        scale = np.exp(rng.uniform(np.log(0.01), np.log(100.0), F)).astype(np.float32)
        beta = (rng.normal(0.0, 1.0, F) / (scale * 16.0)).astype(np.float32)
        params = torch.empty(n * (F + 1) + 3, dtype=torch.float32, device="cuda")
        rows = params[: n * (F + 1)].view(n, F + 1)
        g = torch.Generator(device="cuda")
        g.manual_seed(0)
        sc = torch.from_numpy(scale).cuda()
        bt = torch.from_numpy(beta).cuda()
        for r0 in range(0, n, 1 << 20):
            r1 = min(n, r0 + (1 << 20))
            x = torch.randn(r1 - r0, F, device="cuda", generator=g) * sc
            z = torch.randn(r1 - r0, 5, device="cuda", generator=g)
            t4 = z[:, 0] / torch.sqrt((z[:, 1:] ** 2).sum(dim=1) / 4.0)
            rows[r0:r1, :F] = x
            rows[r0:r1, F] = x @ bt + 0.5 * t4
        params[n * (F + 1):] = torch.tensor([4.0, 10.0, 1.0], device="cuda")
        torch.cuda.synchronize()
        return dict(model=M.robust_t_model(F), fast="tensor", forms=("tensor", "gemm", "plain"),
                    params=params, walkers=4096,
                    burn=2, run=10, bins=128, plain_burn=1, plain_run=10, rows=n,
                    row_len=F + 1, hyper_len=3, plain_rows=1 << 16,
                    init=lambda s, seed: s.init_position_normal(seed, 0.0, 0.01),
                    flop=2 * F * n, bytes=4 * (F + 1) * n // (4096 // 2),
                    desc="robust regression, Student-t(4) residuals, X 16,777,216 x 256 with "
                         "column scales log-U[0.01,100], D=257")
    raise ValueError(name)


def run_config(args):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from bayadera_gb300 import _native
    from bayadera_gb300.engine import GB300BayaderaFactory
    torch.cuda.set_device(0)
    wl = _workload(args.config, args.rows)
    if args.rows:
        wl["desc"] += " [profiling case: %d rows]" % args.rows
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    f = GB300BayaderaFactory(device=0, wgs=1024, stream=stream.cuda_stream)
    W = wl["walkers"]
    cur = {}

    def job(s, seed):
        s.init(seed)
        wl["init"](s, seed + 1)
        s.burn_in(cur["B"], 2.0)
        res = s.run_sampler(cur["R"], 2.0)
        s.mean()
        s.variance()
        s.histogram(1, wl["bins"])
        return res

    out = {}
    kinds = {"tensor": dict(form="gemm", tensor=True), "gemm": dict(form="gemm"),
             "tiled": dict(form="tiled"), "plain": dict(form="plain")}
    forms = wl.get("forms", (wl["fast"], "plain"))
    if args.forms:
        forms = tuple(args.forms.split(","))
    for form in forms:
        sf = f.mcmc_factory(wl["model"], **kinds[form])
        params = wl["params"]
        plain_rows = None
        if form == "plain" and wl.get("plain_rows"):
            # One thread per walker loops over every row, so the plain form's cost is
            # linear in the rows; it is measured on the first plain_rows rows (at full size
            # a job would take many minutes, and C5's 4.3e9-float data exceeds the uint32
            # data length of the reference's model ABI) and scaled to the full row count.
            plain_rows = wl["plain_rows"]
            F1 = wl["row_len"]
            nh = wl["hyper_len"]
            params = torch.cat([params[: plain_rows * F1], params[-nh:]])
        s = sf.create_sampler(11, W, params)
        steps = args.steps if form == wl["fast"] else 1
        B = wl["burn"] if form == wl["fast"] else wl.get("plain_burn", wl["burn"])
        R = wl["run"] if form == wl["fast"] else wl.get("plain_run", wl["run"])
        cur["B"], cur["R"] = B, R
        for w in range(args.warmup if form == wl["fast"] else 1):
            job(s, 100 + w)
        torch.cuda.synchronize()
        times = []
        l0 = _native.launch_count()
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xff)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = job(s, 1000 + 17 * k)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        launches = _native.launch_count() - l0
        # bare-move probe: average time per ensemble step
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        nprobe = max(1, min(B, 8))
        e0.record(stream)
        s.burn_in(nprobe, 2.0)
        e1.record(stream)
        e1.synchronize()
        t_step = e0.elapsed_time(e1) / 1e3 / nprobe
        scale = (plain_rows / wl["rows"]) if plain_rows else 1.0
        out[form] = {"value": W * (B + R) * steps / sum(times) * scale,
                     "ms_per_job": 1e3 * sum(times) / steps,
                     "launches": launches, "ms_per_ensemble_step": 1e3 * t_step,
                     "fp32_tflops_per_step": W * wl["flop"] * scale / t_step / 1e12,
                     "acceptance_rate": res["acceptance_rate"]}
        if plain_rows is not None:
            out[form]["rows_measured"] = plain_rows
            out[form]["value_measured"] = out[form]["value"] / scale
        s.release()
        sf.release()
        del params
    if wl["fast"] not in out or "plain" not in out:
        print(json.dumps({"config": wl["desc"], "forms": out}))
        f.release()
        return 0
    fast = out[wl["fast"]]
    B, R = wl["burn"], wl["run"]
    line = {"metric": "walker-steps/s", "value": fast["value"], "unit": "walker-steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": fast["ms_per_job"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": wl["desc"], "walkers": W, "burn_in": B, "run": R,
                       "form": wl["fast"], "l2": "flushed between timed jobs"},
            "forms": dict({k: v for k, v in out.items() if k != "plain"},
                          plain_fp32=out["plain"],
                          speedup_vs_plain=fast["value"] / out["plain"]["value"]),
            "algorithmic": {"flop_per_walker_step": wl["flop"],
                            "bytes_per_walker_step": wl["bytes"]}}
    print(json.dumps(line))
    f.release()
    return 0


# ------------------------------------------------------------------ batched models
def c4_members(M, n=512, seed=0):
    """512 Gaussian hierarchical models: J log-uniform in [2, 128] groups (dimension
    J + 2), n_j log-uniform in [10, 1000] observations per group, sigma_j log-uniform in
    [0.5, 2] (known), theta_j ~ N(mu, tau^2) with mu ~ N(0, 3^2), log tau ~ N(0, 0.5^2);
    walkers per model from {256, 512, 1024, 4096}; seeded."""
    rng = np.random.default_rng(seed)
    out = []
    for m in range(n):
        J = int(round(np.exp(rng.uniform(np.log(2.0), np.log(128.0)))))
        nj = np.round(np.exp(rng.uniform(np.log(10.0), np.log(1000.0), J))).astype(int)
        sig = np.exp(rng.uniform(np.log(0.5), np.log(2.0), J))
        mu, tau = rng.normal(0.0, 3.0), np.exp(rng.normal(0.0, 0.5))
        theta = rng.normal(mu, tau, J)
        ys = [rng.normal(theta[j], sig[j], nj[j]) for j in range(J)]
        params, rows = M.hierarchical_rows_params(ys, sig)
        W = int(rng.choice([256, 512, 1024, 4096]))
        out.append({"dim": J + 2, "seed": 1000 + m, "walkers": W, "params": params,
                    "rows": rows})
    return out


def run_c4(args):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    from bayadera_gb300 import _native
    from bayadera_gb300 import models as M
    from bayadera_gb300.engine import GB300BayaderaFactory
    torch.cuda.set_device(0)
    BURN4, RUN4 = 1000, 2000
    mem = c4_members(M)
    W = np.array([m["walkers"] for m in mem], np.float64)
    N = np.array([m["rows"] for m in mem], np.float64)
    J = np.array([m["dim"] - 2 for m in mem], np.float64)
    flop_step = float(np.sum(W * (3 * N + 3 * J)))
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    f = GB300BayaderaFactory(device=0, wgs=1024, stream=stream.cuda_stream)
    fam = f.mcmc_factory(M.hierarchical_rows_batch_model(128), form="batch")
    b = fam.create_batch(mem)
    seeds = [7 + i for i in range(len(mem))]

    def job(k):
        b.init_position_normal([s + 31 * k for s in seeds], 0.0, 1.0)
        b.burn_in(BURN4, 2.0)
        return b.run_sampler(RUN4, 2.0)

    for w in range(args.warmup):
        job(100 + w)
    torch.cuda.synchronize()
    times = []
    l0 = _native.launch_count()
    with ClockSampler(0) as clocks:
        for k in range(args.steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xff)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            res = job(k)
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
    launches = _native.launch_count() - l0
    # one burn-in step alone: time per ensemble step of the whole batch
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    b.burn_in(64, 2.0)
    e1.record(stream)
    e1.synchronize()
    t_step = e0.elapsed_time(e1) / 1e3 / 64
    info = b.info()
    b.release()
    fam.release()
    value = float(np.sum(W)) * (BURN4 + RUN4) * args.steps / sum(times)

    # plain single-model form: a uniform random sample of the members, each its own
    # sampler (one plain kernel per half-step, the reference's structure), run in turn;
    # the full job's time is estimated as (members / sample) x the sample's time
    rng = np.random.default_rng(1)
    sample = sorted(rng.choice(len(mem), size=16, replace=False).tolist())
    PB, PR = 50, 100
    compiled, t_plain = {}, 0.0
    for i in sample:
        m = mem[i]
        if m["dim"] not in compiled:
            compiled[m["dim"]] = f.mcmc_factory(M.hierarchical_rows_model(m["dim"] - 2),
                                                form="plain")
        s = compiled[m["dim"]].create_sampler(m["seed"], m["walkers"], m["params"])
        s.init_position_normal(seeds[i], 0.0, 1.0)
        s.burn_in(5, 2.0)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        s.burn_in(PB, 2.0)
        s.run_sampler(PR, 2.0)
        e1.record(stream)
        e1.synchronize()
        t_plain += e0.elapsed_time(e1) / 1e3 * (BURN4 + RUN4) / (PB + PR)
        s.release()
    for sf in compiled.values():
        sf.release()
    f.release()
    t_plain_full = t_plain * len(mem) / len(sample)
    plain_value = float(np.sum(W)) * (BURN4 + RUN4) / t_plain_full
    fp32_peak = 152 * 128 * 2 * 2.07e9 / 1e12
    achieved = flop_step / t_step / 1e12
    rates = res["acceptance_rates"]
    line = {"metric": "walker-steps/s", "value": value, "unit": "walker-steps/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded)",
            "config": {"workload": "512 Gaussian hierarchical models, J log-U[2,128], n_j "
                                   "log-U[10,1000], walkers {256,512,1024,4096}",
                       "models": len(mem), "walkers_total": int(np.sum(W)),
                       "rows_total": int(np.sum(N)), "burn_in": BURN4, "run": RUN4,
                       "form": "batch (3 launches per half-step over balanced work lists, "
                               "CUDA-graph chunks)",
                       "rows_items_per_half_step": info["items"],
                       "l2": "flushed between timed jobs"},
            "gpu_launches": launches,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": fp32_peak,
                         "unit": "TFLOP/s", "frac": achieved / fp32_peak,
                         "peak_kind": "nominal (152 SMs x 128 FMA lanes x 2.07 GHz)",
                         "ms_per_ensemble_step": 1e3 * t_step,
                         "flop_per_ensemble_step": flop_step},
            "forms": {"batch": value, "plain_fp32": plain_value,
                      "speedup_vs_plain": value / plain_value,
                      "plain_sample": "%d of %d members, %d+%d steps each, time scaled to the "
                                      "full job" % (len(sample), len(mem), PB, PR)},
            "clocks": clocks.summary(),
            "result": {"acceptance_rate_min": float(rates.min()),
                       "acceptance_rate_max": float(rates.max())}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ GPU arm
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2 (default): the 50-D Gaussian job; c1, c3, c5: the other "
                         "benchmark workloads, measured GEMM/tiled form vs plain form")
    ap.add_argument("--rows", type=int, default=0,
                    help="with --config c3 or c5: data rows instead of the configuration's "
                         "(a smaller case for profiling); the line then names the row count")
    ap.add_argument("--forms", default="",
                    help="with --config: comma-separated subset of the forms to run "
                         "(tensor, gemm, tiled, plain), e.g. for a profile of one form")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == "c4":
        return run_c4(args)
    if args.config != "c2":
        return run_config(args)

    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    import __graft_entry__
    __graft_entry__.build()
    from bayadera_gb300 import _native
    from bayadera_gb300 import models as M
    from bayadera_gb300.engine import GB300BayaderaFactory

    stream = torch.cuda.Stream()
    P, sigma = precision_matrix()
    dP = torch.from_numpy(P.reshape(-1).copy()).cuda()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    f = GB300BayaderaFactory(device=local, wgs=1024, stream=stream.cuda_stream)
    model = M.mvn_precision_model(DIM)
    sfs = {"tensor": f.mcmc_factory(model, form="gemm", tensor=True),
           "gemm": f.mcmc_factory(model, form="gemm"),
           "plain": f.mcmc_factory(model, form="plain")}
    seed_base = 1000 * (rank + 1)

    def job(samp, seed):
        samp.init(seed)
        samp.init_position_normal(seed + 1)
        samp.burn_in(BURN, 2.0)
        res = samp.run_sampler(RUN, 2.0)
        mean = samp.mean()
        var = samp.variance()
        hist = samp.histogram(1, BINS)
        return res, mean, var, hist

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    def timed_jobs(samp, steps, warmup):
        """Warm-up jobs, then `steps` jobs each timed with CUDA events on the library's
        stream, the L2 flushed by a 256 MiB write before each (outside the events)."""
        for w in range(warmup):
            job(samp, seed_base + 10 * w)
        torch.cuda.synchronize()
        times, results = [], None
        barrier()
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xff)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            results = job(samp, seed_base + 7919 * (k + 1))
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
        barrier()
        t_total = max_over_ranks(sum(times), dist, "cuda")
        return replica_throughput(steps, world, t_total), t_total, results

    # headline: the GEMM form on the tensor cores (64-walker tiles, x'Px as a split-bf16
    # tcgen05 product against the resident precision matrix)
    samp = sfs["tensor"].create_sampler(seed_base, WALKERS, dP)
    launches0 = _native.launch_count()
    with ClockSampler(local) as clocks:
        value, t_total, results = timed_jobs(samp, args.steps, args.warmup)
    launches = _native.launch_count() - launches0

    # the fp32 SIMT GEMM form (64-walker tiles, register-blocked x'Px from shared memory)
    samp_gemm = sfs["gemm"].create_sampler(seed_base, WALKERS, dP)
    gemm_value, _, _ = timed_jobs(samp_gemm, max(1, min(args.steps, 2)), 1)
    samp_gemm.release()

    # the plain FP32 form (one thread per walker, the reference's kernel structure)
    samp_plain = sfs["plain"].create_sampler(seed_base, WALKERS, dP)
    plain_value, _, _ = timed_jobs(samp_plain, max(1, min(args.steps, 2)), 1)
    samp_plain.release()

    # dominant kernel: bare stretch launches of a burn-in, events on the launching stream
    n_probe = 256
    with torch.cuda.stream(stream):
        flush.fill_(1)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    samp.burn_in(n_probe, 2.0)
    e1.record(stream)
    e1.synchronize()
    t_launch = e0.elapsed_time(e1) / 1e3 / (2 * n_probe)
    bytes_launch = (WALKERS // 2) * BYTES_PER_WALKER_STEP
    flop_launch = (WALKERS // 2) * FLOP_PER_WALKER_STEP
    hbm_peak, peak_kind = measured_peaks()
    achieved = bytes_launch / t_launch / 1e9
    traffic = profile_traffic()

    # e2e: the same job through the C ABI from host buffers
    e2e_times = []
    h2d = P.nbytes
    d2h = 0
    for k in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = sfs["tensor"].create_sampler(seed_base + 31 * k, WALKERS, P.reshape(-1))
        res, mean, var, hist = job(s2, seed_base + 31 * k)
        s2.release()
        e2e_times.append(time.perf_counter() - t0)
        d2h = (8 + 3 * DIM * 8 + 2 * DIM * 8 + hist.limits.nbytes + hist.pdf.nbytes
               + hist.bin_ranks.nbytes)
    e2e_value = WALKERS * (BURN + RUN) * world / statistics.median(e2e_times)

    # the job's result: posterior means within 3 MC s.e. of the analytic mean 0
    res, mean, var, hist = results
    ac = res["autocorrelation"]
    within = None
    within_tmax = None
    err_sd = None
    if ac is not None:
        within = int(np.sum(np.abs(ac.mean) <= 3 * ac.sigma))
        # the same test with each dimension's standard error taken at the largest tau of the
        # run (sigma scales with sqrt(tau)): acor's per-dimension tau from n / tau ~ 6
        # correlation times is itself low for some dimensions
        tau = np.asarray(ac.tau, np.float64)
        se_tmax = np.asarray(ac.sigma) * np.sqrt(np.max(tau) / np.maximum(tau, 1e-30))
        within_tmax = int(np.sum(np.abs(ac.mean) <= 3 * se_tmax))
        # the run mean's distance from the analytic mean 0, in posterior standard deviations
        err_sd = float(np.max(np.abs(ac.mean) / np.sqrt(np.diag(sigma))))

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_sample(12.0)

    if rank == 0:
        line = {
            "metric": "walker-steps/s", "value": value, "unit": "walker-steps/s",
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * t_total / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded AR(1) precision matrix, seed 0)",
            "config": config(),
            "e2e": {"value": e2e_value, "unit": "walker-steps/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h},
            "gpu_launches": launches,
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                         "peak_kind": peak_kind,
                         "kernel": "bay_tcr_bare (GEMM form on the tensor cores, resident matrix)",
                         "launch_us": t_launch * 1e6,
                         "fp32_tflops": flop_launch / t_launch / 1e12},
            "cpu_baseline": cpu,
            "forms": {"tensor": value, "gemm_fp32_simt": gemm_value, "plain_fp32": plain_value,
                      "speedup_vs_plain": value / plain_value},
            "clocks": clocks.summary(),
            "result": {"acceptance_rate": res["acceptance_rate"],
                       "tau_max": float(np.max(ac.tau)) if ac is not None else None,
                       "means_within_3se": within,
                       "means_within_3se_at_tau_max": within_tmax, "dims": DIM,
                       "max_abs_mean_over_posterior_sd": err_sd},
        }
        print(json.dumps(line))
    samp.release()
    for x in sfs.values():
        x.release()
    f.release()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
