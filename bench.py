#!/usr/bin/env python
"""Throughput of the ensemble stretch-move engine: walker-steps/s on the 50-dimensional
correlated Gaussian workload (AR(1) covariance, rho = 0.9, per-dimension scales
log-uniform in [0.1, 10], precision matrix as 2500 hyperparameters; 65,536 walkers
initialised N(0, I); 2,000 burn-in and 4,000 sampling steps; outputs mean, variance,
acor and 128-bin histograms).

One step = that whole job on one GPU.  `value` times it with the inputs resident on the
device; `e2e` times the same job through the C ABI from host buffers (sampler creation
with the host copy of the precision matrix, results copied back).  The default line also
carries `configs`: the other benchmark workloads (the 2-D Gaussian posterior, logistic
regression, 512 hierarchical models, robust regression), each its fast form beside the
plain fp32 form with its log-density error against FP64 on its own data.  The reference
arm (--impl reference) times the CPU restatement of the reference's stretch kernel, built
for speed, on the host cores.  Multi-GPU: independent replicas (the path has no exchange
step).
"""
import argparse
import json
import math
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
LOG_SQRT_2PI = 0.5 * math.log(2.0 * math.pi)
# the reference arm and cpu_baseline: the whole 50-D job on this many of its walkers
CPU_WALKERS = 8192


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
    """Roofline denominators: the machine's measured HBM copy bandwidth (GB/s) and cuBLAS bf16
    rate (TFLOP/s, burst), else the stated fallbacks."""
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            j = json.load(f)
        return {"hbm_gbs": float(j.get("hbm_gbs", 6800.0)),
                "bf16_tflops": float(j.get("bf16_tflops", 1900.0)), "kind": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "kind": "fallback"}


FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.07e9 / 1e12     # nominal: no measured FP32 figure


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


# ------------------------------------------------------------------ FP64 error measures
# Log densities of the configs' models in FP64 (numpy, or torch float64 for the large
# design matrices), written from the models' formulas; used to report each config's
# log-density error on its own data.
def _err(lf, want):
    lf = np.asarray(lf, np.float64)
    want = np.asarray(want, np.float64)
    ok = np.isfinite(want)
    err = np.abs(lf[ok] - want[ok])
    rel = err / np.maximum(np.abs(want[ok]), 1e-30)
    return {"max_abs": float(err.max()), "median_abs": float(np.median(err)),
            "max_rel": float(rel.max()), "walkers": int(ok.sum())}


def fp64_c1(params, pos):
    """2-D (mu, sigma) posterior: sum_i log N(y_i | mu, sigma) + log N(mu | h0, h1) +
    log U(sigma | h2, h3); pos (W, 2)."""
    y = np.asarray(params[:-4], np.float64)
    h = np.asarray(params[-4:], np.float64)
    mu, sg = pos[:, 0].astype(np.float64), pos[:, 1].astype(np.float64)
    ss = np.zeros(mu.size)
    for c in range(0, y.size, 2000):
        ss += ((y[None, c:c + 2000] - mu[:, None]) ** 2).sum(axis=1)
    ll = -ss / (2.0 * sg * sg) - y.size * (np.log(sg) + LOG_SQRT_2PI)
    pr = -(mu - h[0]) ** 2 / (2.0 * h[1] ** 2) - math.log(h[1]) - LOG_SQRT_2PI
    pr = pr + np.where((h[2] <= sg) & (sg <= h[3]), -math.log(h[3] - h[2]), -np.inf)
    return ll + pr


def fp64_mvn(P, pos):
    P64 = P.astype(np.float64)
    x = pos.astype(np.float64)
    return -0.5 * np.einsum("wi,ij,wj->w", x, P64, x)


def fp64_logistic(rows_dev, F, sd, pos):
    """sum_n y_n eta_n - softplus(eta_n) - |beta|^2 / (2 sd^2); rows_dev (n, F + 1) on the
    device, summed in torch float64 by row chunks."""
    import torch
    B = torch.from_numpy(pos.astype(np.float64)).cuda()
    acc = torch.zeros(B.shape[0], dtype=torch.float64, device="cuda")
    for r0 in range(0, rows_dev.shape[0], 1 << 18):
        blk = rows_dev[r0:r0 + (1 << 18)].double()
        eta = blk[:, :F] @ B.T
        y = blk[:, F:F + 1]
        acc += (y * eta - (eta.clamp(min=0.0) + torch.log1p(torch.exp(-eta.abs())))).sum(0)
    acc -= (B * B).sum(1) / (2.0 * sd * sd)
    return acc.cpu().numpy()


def fp64_robust_t(rows_dev, F, h, pos):
    """sum_n -(nu + 1)/2 log(1 + r_n^2 / nu) - N log sigma - |beta|^2/(2 h1^2)
    - (log sigma)^2/(2 h2^2), r = (y - x.beta)/sigma; torch float64 by row chunks."""
    import torch
    X = torch.from_numpy(pos.astype(np.float64)).cuda()
    B, ls = X[:, :F], X[:, F]
    inv_s = torch.exp(-ls)
    nu = float(h[0])
    acc = torch.zeros(X.shape[0], dtype=torch.float64, device="cuda")
    n = rows_dev.shape[0]
    for r0 in range(0, n, 1 << 19):
        blk = rows_dev[r0:r0 + (1 << 19)].double()
        z = (blk[:, F:F + 1] - blk[:, :F] @ B.T) * inv_s[None, :]
        acc += (-0.5 * (nu + 1.0) * torch.log1p(z * z / nu)).sum(0)
    acc += -n * ls - (B * B).sum(1) / (2.0 * float(h[1]) ** 2) - ls * ls / (2.0 * float(h[2]) ** 2)
    return acc.cpu().numpy()


def fp64_hrows(params, rows, pos):
    """Row-encoded hierarchical model: sum_i c_i (y_i - theta_g_i)^2 + sum_j [-(theta_j -
    mu)^2/(2 tau^2) - log tau] - mu^2/(2 h0^2) - (log tau)^2/(2 h1^2); pos (W, J + 2)."""
    r = np.asarray(params[:3 * rows], np.float64).reshape(rows, 3)
    h = np.asarray(params[3 * rows:], np.float64)
    x = pos.astype(np.float64)
    J = x.shape[1] - 2
    g = r[:, 1].astype(np.int64)
    d = r[None, :, 0] - x[:, g]
    res = (r[None, :, 2] * d * d).sum(axis=1)
    mu, lt = x[:, J], x[:, J + 1]
    res += (-(x[:, :J] - mu[:, None]) ** 2 * 0.5 * np.exp(-2.0 * lt)[:, None]).sum(axis=1)
    return res - J * lt - mu * mu / (2.0 * h[0] ** 2) - lt * lt / (2.0 * h[1] ** 2)


# ------------------------------------------------------------------ CPU port (reference arm)
def cpu_port(threads, walkers=CPU_WALKERS):
    """The CPU restatement of the reference's stretch kernel plus the same model, in its
    speed build (-O3 -ffast-math -funroll-loops, OpenMP over the walkers of a half-step):
    the reference's own CPU path (OpenCL on pocl) cannot run here."""
    from oracle import oracle as O
    O.use_speed_build(True)
    P, _ = precision_matrix()
    r = O.Stretch("mvn_precision", DIM, walkers, P.reshape(-1), seed=SEED, threads=threads,
                  flags=O.ACCEPT_LOG)
    return O, r


def cpu_job(O, r, seed):
    """The 50-D job on the CPU port: init!, N(0, I) walkers, 2,000 burn-in steps, 4,000
    accu steps with per-step means, mean, variance, 128-bin histograms, acor."""
    r.init(seed)
    r.init_position_normal(seed + 1)
    r.burn_in(BURN, 2.0)
    _, means = r.run_sampler(RUN, 2.0)
    O.mean64(r.xs, DIM)
    O.variance64(r.xs, DIM)
    O.histogram([r.xs], DIM, BINS)
    O.acor64(means)


def cpu_sample(budget_s=10.0):
    """cpu_baseline: whole CPU-port jobs on CPU_WALKERS walkers until budget_s of work."""
    threads = os.cpu_count() or 1
    O, r = cpu_port(threads)
    times = []
    while not times or sum(times) < budget_s:
        t0 = time.perf_counter()
        cpu_job(O, r, SEED + 7 * len(times))
        times.append(time.perf_counter() - t0)
    v = CPU_WALKERS * (BURN + RUN) * len(times) / sum(times)
    return {"value": v, "unit": "walker-steps/s", "cores": threads, "kind": "port",
            "sample": "%d whole 50-D jobs (2,000 burn-in + 4,000 run steps, mean, variance, "
                      "128-bin histograms, acor) on %d of the 65,536 walkers, %.1f s; speed "
                      "build of the CPU port" % (len(times), CPU_WALKERS, sum(times))}


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
    """The reference arm: each step is one whole 50-D job on CPU_WALKERS walkers on the
    host cores (the job's per-walker work does not depend on the walker count; the full
    65,536-walker job would take about 8 x as long per step)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    O, r = cpu_port(threads)
    for w in range(args.warmup):
        cpu_job(O, r, 100 + w)
    times = []
    for k in range(args.steps):
        t0 = time.perf_counter()
        cpu_job(O, r, 1000 + 17 * k)
        times.append(time.perf_counter() - t0)
    t_med = statistics.median(times)
    v = CPU_WALKERS * (BURN + RUN) / t_med
    sample = ("each step one whole 50-D job (2,000 burn-in + 4,000 run steps, mean, "
              "variance, 128-bin histograms, acor) on %d of the 65,536 walkers; median of %d "
              "steps; speed build of the CPU port (-O3 -ffast-math, OpenMP)"
              % (CPU_WALKERS, args.steps))
    line = {
        "impl": "reference", "metric": "walker-steps/s", "value": v, "unit": "walker-steps/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * t_med, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(config(), cpu_walkers=CPU_WALKERS),
        "cpu_baseline": {"value": v, "unit": "walker-steps/s", "cores": threads,
                         "kind": "port", "sample": sample},
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
def _workload(name, rows=0, quick=False):
    """Model, params, walkers, steps, init, algorithmic work and FP64 error measure of the
    benchmark workloads other than the 50-D job.  quick: fewer plain-form steps (the
    configs object of the default line)."""
    import torch
    from bayadera_gb300 import models as M
    if name == "c1":
        rng = np.random.default_rng(0)
        data = rng.normal(3.0, 2.0, 10000).astype(np.float32)
        params = np.concatenate([data, np.array([0.0, 10.0, 0.0, 20.0], np.float32)])
        return dict(model=M.gaussian_posterior_model(), fast="tiled", params=params,
                    walkers=4096, burn=512, run=1024, bins=256,
                    init=lambda s, seed: s.init_position(seed, [2.0, 4.0, 1.0, 3.0]),
                    flop=3 * 10000, bytes=0, bound="fp32",
                    fp64=lambda pos: fp64_c1(params, pos), check=4096,
                    desc="2-D Gaussian (mu, sigma) posterior, N=10,000 data, prior "
                         "N(0,10^2) x U(0,20)")
    if name == "c3":
        n, F = rows or (1 << 20), 64
        rng = np.random.default_rng(0)
        X = rng.standard_normal((n, F), dtype=np.float32)
        beta = rng.normal(0.0, 1.0 / 8.0, F)
        eta = X.astype(np.float64) @ beta
        y = (rng.random(n) < 1.0 / (1.0 + np.exp(-eta))).astype(np.float32)
        rws = np.empty((n, F + 1), np.float32)
        rws[:, :F] = X
        rws[:, F] = y
        params = torch.from_numpy(np.concatenate([rws.reshape(-1), [5.0]]).astype(np.float32)).cuda()
        rows_dev = params[: n * (F + 1)].view(n, F + 1)
        return dict(model=M.logistic_model(F), fast="tensor", forms=("tensor", "gemm", "plain"),
                    params=params, walkers=8192,
                    burn=10, run=20, bins=128, plain_burn=1, plain_run=4, rows=n,
                    row_len=F + 1, hyper_len=1, plain_rows=(1 << 16) if quick else 0,
                    init=lambda s, seed: s.init_position_normal(seed, 0.0, 0.05),
                    flop=2 * F * n, bytes=4 * (F + 1) * n // (8192 // 2), bound="tensor",
                    fp64=lambda pos: fp64_logistic(rows_dev, F, 5.0, pos), check=256,
                    desc="Bayesian logistic regression, X 1,048,576 x 64 N(0,1), beta* ~ "
                         "N(0,1/64), prior N(0,5^2 I)")
    if name == "c5":
        n, F = rows or (1 << 24), 256
        rng = np.random.default_rng(0)
        scale = np.exp(rng.uniform(np.log(0.01), np.log(100.0), F)).astype(np.float32)
        beta = (rng.normal(0.0, 1.0, F) / (scale * 16.0)).astype(np.float32)
        params = torch.empty(n * (F + 1) + 3, dtype=torch.float32, device="cuda")
        rws = params[: n * (F + 1)].view(n, F + 1)
        g = torch.Generator(device="cuda")
        g.manual_seed(0)
        sc = torch.from_numpy(scale).cuda()
        bt = torch.from_numpy(beta).cuda()
        for r0 in range(0, n, 1 << 20):
            r1 = min(n, r0 + (1 << 20))
            x = torch.randn(r1 - r0, F, device="cuda", generator=g) * sc
            z = torch.randn(r1 - r0, 5, device="cuda", generator=g)
            t4 = z[:, 0] / torch.sqrt((z[:, 1:] ** 2).sum(dim=1) / 4.0)
            rws[r0:r1, :F] = x
            rws[r0:r1, F] = x @ bt + 0.5 * t4
        hyper = np.array([4.0, 10.0, 1.0], np.float32)
        params[n * (F + 1):] = torch.from_numpy(hyper).cuda()
        torch.cuda.synchronize()
        return dict(model=M.robust_t_model(F), fast="tensor", forms=("tensor", "gemm", "plain"),
                    params=params, walkers=4096,
                    burn=2, run=10, bins=128, plain_burn=1, plain_run=4 if quick else 10,
                    rows=n, row_len=F + 1, hyper_len=3, plain_rows=1 << 16,
                    init=lambda s, seed: s.init_position_normal(seed, 0.0, 0.01),
                    flop=2 * F * n, bytes=4 * (F + 1) * n // (4096 // 2), bound="tensor",
                    fp64=lambda pos: fp64_robust_t(rws, F, hyper, pos), check=64,
                    desc="robust regression, Student-t(4) residuals, X 16,777,216 x 256 with "
                         "column scales log-U[0.01,100], D=257")
    raise ValueError(name)


def _roofline(bound, flop, bytes_, t_step, W, peaks):
    """Roofline entry of a config: algorithmic work per ensemble step over its measured
    time against the bound's peak (measured HBM or bf16; nominal FP32)."""
    if bound == "fp32":
        a = W * flop / t_step / 1e12
        return {"bound": "fp32", "achieved": a, "peak": FP32_PEAK_TFLOPS, "unit": "TFLOP/s",
                "frac": a / FP32_PEAK_TFLOPS, "peak_kind": "nominal (152 SMs x 128 FMA lanes x "
                                                            "2.07 GHz)"}
    if bound == "tensor":
        a = W * flop / t_step / 1e12
        return {"bound": "tensor", "achieved": a, "peak": peaks["bf16_tflops"], "unit": "TFLOP/s",
                "frac": a / peaks["bf16_tflops"], "peak_kind": peaks["kind"] + " bf16 (burst)",
                "note": "algorithmic 2 F N per walker-step; the split form issues 3 bf16 "
                        "products, so the tensor pipe carries 3 x this",
                "hbm_gbs_algorithmic": W * bytes_ / t_step / 1e9}
    a = W * bytes_ / t_step / 1e9
    return {"bound": "hbm", "achieved": a, "peak": peaks["hbm_gbs"], "unit": "GB/s",
            "frac": a / peaks["hbm_gbs"], "peak_kind": peaks["kind"]}


def measure_config(name, steps, warmup, rows=0, forms=None, quick=False, factory=None):
    """Times the workload's fast form (and the plain fp32 form, and for the regressions the
    fp32 SIMT GEMM form unless quick) on whole jobs, the L2 flushed before each; returns
    the config's record."""
    import torch
    from bayadera_gb300 import _native
    from bayadera_gb300.engine import GB300BayaderaFactory
    wl = _workload(name, rows, quick)
    if rows:
        wl["desc"] += " [profiling case: %d rows]" % rows
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
    forms = forms or wl.get("forms", (wl["fast"], "plain"))
    if quick:
        forms = tuple(x for x in forms if x != "gemm")
    err = None
    # the fast form's kernel shape, chosen by the library's autotuner on this workload
    tune = tuned(lambda: f.autotune(wl["model"], W, wl["params"], **kinds[wl["fast"]]))
    for form in forms:
        shape = tune["shape"] if form == wl["fast"] else {}
        sf = f.mcmc_factory(wl["model"], **kinds[form], **shape)
        params = wl["params"]
        plain_rows = None
        if form == "plain" and wl.get("plain_rows"):
            # One thread per walker loops over every row, so the plain form's cost is
            # linear in the rows; it is measured on the first plain_rows rows and scaled to
            # the full row count (at full size a job takes minutes, and C5's 4.3e9-float
            # data exceeds the uint32 data length of the reference's model ABI).
            plain_rows = wl["plain_rows"]
            params = torch.cat([params[: plain_rows * wl["row_len"]], params[-wl["hyper_len"]:]])
        s = graphs(sf.create_sampler(11, W, params))
        fast = form == wl["fast"]
        n_steps = steps if fast else 1
        B = wl["burn"] if fast else wl.get("plain_burn", wl["burn"])
        R = wl["run"] if fast else wl.get("plain_run", wl["run"])
        cur["B"], cur["R"] = B, R
        for w in range(warmup if fast else 1):
            job(s, 100 + w)
        torch.cuda.synchronize()
        times = []
        l0 = _native.launch_count()
        for k in range(n_steps):
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
        if fast:
            pos = s.positions().T
            lf = s.logfn()
            idx = np.linspace(0, W - 1, min(W, wl["check"])).astype(np.int64)
            err = _err(lf[idx], wl["fp64"](pos[idx]))
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
        out[form] = {"value": W * (B + R) * n_steps / sum(times) * scale,
                     "ms_per_job": 1e3 * sum(times) / n_steps / scale,
                     "launches": launches, "ms_per_ensemble_step": 1e3 * t_step / scale,
                     "acceptance_rate": res["acceptance_rate"]}
        if plain_rows is not None:
            out[form]["rows_measured"] = plain_rows
            out[form]["value_measured"] = out[form]["value"] / scale
        s.release()
        sf.release()
        del params
    f.release()
    fast = out[wl["fast"]]
    rec = {"workload": wl["desc"], "walkers": W, "burn_in": wl["burn"], "run": wl["run"],
           "form": wl["fast"], "value": fast["value"], "unit": "walker-steps/s",
           "ms_per_job": fast["ms_per_job"], "gpu_launches": fast["launches"],
           "acceptance_rate": fast["acceptance_rate"],
           "roofline": _roofline(wl["bound"], wl["flop"], wl["bytes"],
                                 fast["ms_per_ensemble_step"] / 1e3, W, measured_peaks()),
           "logfn_err_vs_fp64": err,
           "autotune": tune,
           "forms": {k: v for k, v in out.items()},
           "algorithmic": {"flop_per_walker_step": wl["flop"],
                           "bytes_per_walker_step": wl["bytes"]}}
    if "plain" in out:
        rec["plain_fp32"] = out["plain"]["value"]
        rec["speedup_vs_plain"] = fast["value"] / out["plain"]["value"]
        if "rows_measured" in out["plain"]:
            rec["plain_fp32_note"] = ("measured on the first %d rows, scaled to the full row "
                                      "count (cost linear in the rows)"
                                      % out["plain"]["rows_measured"])
    return rec


def run_config(args):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    torch.cuda.set_device(0)
    forms = tuple(args.forms.split(",")) if args.forms else None
    with ClockSampler(0) as clocks:
        rec = measure_config(args.config, args.steps, args.warmup, args.rows, forms)
    line = {"metric": "walker-steps/s", "value": rec["value"], "unit": "walker-steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": rec["ms_per_job"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {"workload": rec["workload"], "walkers": rec["walkers"],
                       "burn_in": rec["burn_in"], "run": rec["run"], "form": rec["form"],
                       "l2": "flushed between timed jobs"},
            "gpu_launches": rec["gpu_launches"], "roofline": rec["roofline"],
            "logfn_err_vs_fp64": rec["logfn_err_vs_fp64"], "forms": rec["forms"],
            "autotune": rec["autotune"], "clocks": clocks.summary()}
    for k in ("plain_fp32", "speedup_vs_plain", "plain_fp32_note"):
        if k in rec:
            line[k] = rec[k]
    if NO_GRAPHS:
        line["config"]["graphs"] = "off (--no-graphs: kernels launched one by one)"
    print(json.dumps(line))
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


def measure_c4(steps, warmup, members=512, plain=True):
    """The 512-model batch: whole jobs (init, 1,000 burn-in and 2,000 accu steps of every
    member) timed with the L2 flushed before each, the plain single-model form on a sample
    of the members (unless plain is False); returns the config's record."""
    import torch
    from bayadera_gb300 import _native
    from bayadera_gb300 import models as M
    from bayadera_gb300.engine import GB300BayaderaFactory
    BURN4, RUN4 = 1000, 2000
    mem = c4_members(M, members)
    W = np.array([m["walkers"] for m in mem], np.float64)
    N = np.array([m["rows"] for m in mem], np.float64)
    J = np.array([m["dim"] - 2 for m in mem], np.float64)
    flop_step = float(np.sum(W * (3 * N + 3 * J)))
    stream = torch.cuda.Stream()
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device="cuda")
    f = GB300BayaderaFactory(device=0, wgs=1024, stream=stream.cuda_stream)
    fam = f.mcmc_factory(M.hierarchical_rows_batch_model(128), form="batch")
    tune = tuned(lambda: fam.autotune_batch(mem))   # the work lists' shape, by timing (untimed)
    b = graphs(fam.create_batch(mem, tune["shape"]))
    seeds = [7 + i for i in range(len(mem))]

    def job(k):
        b.init_position_normal([s + 31 * k for s in seeds], 0.0, 1.0)
        b.burn_in(BURN4, 2.0)
        return b.run_sampler(RUN4, 2.0)

    def timed(persistent):
        """warm-up and timed jobs in one launch mode: three launches per half-step, or one
        persistent launch per chunk of steps"""
        b.set_persistent(persistent)
        for w in range(warmup):
            job(100 + w)
        torch.cuda.synchronize()
        ts = []
        l0 = _native.launch_count()
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xff)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = job(k)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1) / 1e3)
        return ts, _native.launch_count() - l0, r

    def fp64_errors():
        """FP64 error of the members' log densities after the last job (8 members, 64
        walkers each)"""
        errs = []
        pos_all, lf_all = b.positions(), b.logfn()
        for i in np.linspace(0, len(mem) - 1, 8).astype(int):
            m = mem[i]
            idx = np.linspace(0, m["walkers"] - 1, 64).astype(np.int64)
            errs.append(_err(lf_all[i][idx], fp64_hrows(m["params"], m["rows"], pos_all[i][idx])))
        return {"max_abs": max(e["max_abs"] for e in errs),
                "median_abs": float(np.median([e["median_abs"] for e in errs])),
                "max_rel": max(e["max_rel"] for e in errs),
                "walkers": sum(e["walkers"] for e in errs), "members": 8}

    # each launch mode's jobs, each checked against FP64 after its last job
    t_launch, l_launch, res_launch = timed(False)
    err_launch = fp64_errors()
    t_persist, l_persist, res_persist = timed(True)
    err_persist = fp64_errors()
    persistent = sum(t_persist) < sum(t_launch)
    times, launches, res = ((t_persist, l_persist, res_persist) if persistent
                            else (t_launch, l_launch, res_launch))
    b.set_persistent(persistent)
    err = dict(err_persist if persistent else err_launch)
    err["other_launch_mode_max_rel"] = (err_launch if persistent else err_persist)["max_rel"]
    # time per ensemble step of the whole batch
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
    value = float(np.sum(W)) * (BURN4 + RUN4) * steps / sum(times)

    # plain single-model form: a uniform random sample of the members, each its own
    # sampler (one plain kernel per half-step, the reference's structure), run in turn;
    # the full job's time is estimated as (members / sample) x the sample's time
    rng = np.random.default_rng(1)
    sample = sorted(rng.choice(len(mem), size=16, replace=False).tolist()) if plain else []
    PB, PR = 50, 100
    compiled, t_plain = {}, 0.0
    for i in sample:
        m = mem[i]
        if m["dim"] not in compiled:
            compiled[m["dim"]] = f.mcmc_factory(M.hierarchical_rows_model(m["dim"] - 2),
                                                form="plain")
        s = graphs(compiled[m["dim"]].create_sampler(m["seed"], m["walkers"], m["params"]))
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
    plain_value = (float(np.sum(W)) * (BURN4 + RUN4) / (t_plain * len(mem) / len(sample))
                   if sample else None)
    achieved = flop_step / t_step / 1e12
    rates = res["acceptance_rates"]
    return {"workload": "%d Gaussian hierarchical models, J log-U[2,128], n_j log-U[10,1000], "
                        "walkers {256,512,1024,4096}%s"
                        % (len(mem), "" if members == 512 else " [profiling case: the first %d of 512]"
                           % members),
            "models": len(mem), "walkers_total": int(np.sum(W)), "rows_total": int(np.sum(N)),
            "burn_in": BURN4, "run": RUN4,
            "form": "batch (CUDA-graph chunks over balanced work lists; %s)"
                    % ("one persistent launch per chunk" if persistent
                       else "three launches per half-step"),
            "launch_modes_ms_per_job": {"three_launches_per_half_step": 1e3 * sum(t_launch) / steps,
                                        "persistent_per_chunk": 1e3 * sum(t_persist) / steps},
            "rows_items_per_half_step": info["items"],
            "value": value, "unit": "walker-steps/s", "ms_per_job": 1e3 * sum(times) / steps,
            "gpu_launches": launches,
            "roofline": {"bound": "fp32", "achieved": achieved, "peak": FP32_PEAK_TFLOPS,
                         "unit": "TFLOP/s", "frac": achieved / FP32_PEAK_TFLOPS,
                         "peak_kind": "nominal (152 SMs x 128 FMA lanes x 2.07 GHz)",
                         "ms_per_ensemble_step": 1e3 * t_step,
                         "flop_per_ensemble_step": flop_step},
            "logfn_err_vs_fp64": err, "autotune": tune,
            "plain_fp32": plain_value,
            "speedup_vs_plain": value / plain_value if plain_value else None,
            "plain_fp32_note": "%d of %d members, %d+%d steps each, time scaled to the full "
                               "job" % (len(sample), len(mem), PB, PR),
            "acceptance_rate_min": float(rates.min()), "acceptance_rate_max": float(rates.max())}


def run_c4(args):
    import torch
    import __graft_entry__
    __graft_entry__.build()
    torch.cuda.set_device(0)
    with ClockSampler(0) as clocks:
        rec = measure_c4(args.steps, args.warmup, args.members,
                         plain=not args.forms or "plain" in args.forms.split(","))
    line = {"metric": "walker-steps/s", "value": rec["value"], "unit": "walker-steps/s",
            "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": rec["ms_per_job"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
            "config": {k: rec[k] for k in ("workload", "models", "walkers_total", "rows_total",
                                           "burn_in", "run", "form",
                                           "rows_items_per_half_step", "launch_modes_ms_per_job")},
            "gpu_launches": rec["gpu_launches"], "roofline": rec["roofline"],
            "logfn_err_vs_fp64": rec["logfn_err_vs_fp64"], "autotune": rec["autotune"],
            "forms": {"batch": rec["value"], "plain_fp32": rec["plain_fp32"],
                      "speedup_vs_plain": rec["speedup_vs_plain"],
                      "plain_sample": rec["plain_fp32_note"]},
            "clocks": clocks.summary()}
    line["config"]["l2"] = "flushed between timed jobs"
    if NO_GRAPHS:
        line["config"]["graphs"] = "off (--no-graphs: kernels launched one by one)"
    print(json.dumps(line))
    return 0


def measure_configs():
    """The configs object of the default line: the other workloads, each its fast form on
    whole jobs (one warm-up, one or two timed) beside the plain fp32 form, with the
    log-density error against FP64 on the config's own data."""
    import torch
    out = {}
    for name, steps in (("c1", 2), ("c3", 1), ("c5", 1)):
        try:
            out[name] = measure_config(name, steps, 1, quick=True)
        except Exception as e:          # a failed config is reported, not fatal
            out[name] = {"error": repr(e)}
        torch.cuda.empty_cache()
    try:
        out["c4"] = measure_c4(1, 1)
    except Exception as e:
        out["c4"] = {"error": repr(e)}
    return out


# ------------------------------------------------------------------ GPU arm
SHAPE = None   # --shape: a kernel shape given on the command line instead of the autotuner's
NO_GRAPHS = False   # --no-graphs: every kernel launched on its own (for profiles)


def graphs(sampler):
    """The sampler or batch, with CUDA-graph chunks switched off under --no-graphs (ncu
    profiled kernels launched on their own, but none of these graphs' kernel nodes)."""
    if NO_GRAPHS:
        sampler.set_graphs(False)
    return sampler


def tuned(run_tuner):
    """The autotuner's record for the fast form, or, with --shape, the given shape (the
    tuner then does not run: a profile of one shape captures no tuning launches)."""
    if SHAPE is not None:
        return {"shape": dict(SHAPE), "given": True}
    return run_tuner()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-configs", action="store_true",
                    help="default line without the configs object (the other workloads)")
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c3", "c4", "c5"],
                    help="c2 (default): the 50-D Gaussian job; c1, c3, c4, c5: the other "
                         "benchmark workloads, their fast form vs the plain form")
    ap.add_argument("--rows", type=int, default=0,
                    help="with --config c3 or c5: data rows instead of the configuration's "
                         "(a smaller case for profiling); the line then names the row count")
    ap.add_argument("--members", type=int, default=512,
                    help="with --config c4: the first N of the 512 models (a smaller case for "
                         "profiling); the line then names the count")
    ap.add_argument("--forms", default="",
                    help="with --config: comma-separated subset of the forms to run "
                         "(tensor, gemm, tiled, plain), e.g. for a profile of one form")
    ap.add_argument("--shape", default="",
                    help="JSON kernel shape for the fast form, e.g. '{\"tc_groups\": 1}', "
                         "used instead of the autotuner's choice (for profiles of one shape)")
    ap.add_argument("--no-graphs", action="store_true",
                    help="launch every kernel on its own instead of in CUDA-graph chunks (for "
                         "ncu, which profiled none of these graphs' kernel nodes)")
    args = ap.parse_args()
    global SHAPE, NO_GRAPHS
    SHAPE = json.loads(args.shape) if args.shape else None
    NO_GRAPHS = args.no_graphs
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
    # the resident tensor-core kernels' shape (tile groups per CTA), chosen by the library's
    # autotuner on this workload before anything is timed
    tune = tuned(lambda: f.autotune(model, WALKERS, dP, form="gemm", tensor=True))
    sfs = {"tensor": f.mcmc_factory(model, form="gemm", tensor=True, **tune["shape"]),
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
        stream, the L2 flushed by a 256 MiB write before each (outside the events).
        Returns the throughput, the time and every timed job's result."""
        for w in range(warmup):
            job(samp, seed_base + 10 * w)
        torch.cuda.synchronize()
        times, results = [], []
        barrier()
        for k in range(steps):
            with torch.cuda.stream(stream):
                flush.fill_(k & 0xff)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            r = job(samp, seed_base + 7919 * (k + 1))
            e1.record(stream)
            e1.synchronize()
            times.append(e0.elapsed_time(e1) / 1e3)
            results.append(r)
        barrier()
        t_total = max_over_ranks(sum(times), dist, "cuda")
        return replica_throughput(steps, world, t_total), t_total, results

    # headline: the GEMM form on the tensor cores (64-walker tiles, x'Px as a split-bf16
    # tcgen05 product against the resident precision matrix)
    samp = graphs(sfs["tensor"].create_sampler(seed_base, WALKERS, dP))
    launches0 = _native.launch_count()
    with ClockSampler(local) as clocks:
        value, t_total, results = timed_jobs(samp, args.steps, args.warmup)
    launches = _native.launch_count() - launches0
    # log-density error of the last job's walkers against FP64 (the AR(1) matrix itself)
    pos = samp.positions().T
    idx = np.arange(0, WALKERS, 8)
    err = _err(samp.logfn()[idx], fp64_mvn(P, pos[idx]))

    # the comparison forms (--forms tensor skips them: a shorter run for profiling)
    gemm_value = plain_value = None
    only = set(args.forms.split(",")) if args.forms else {"tensor", "gemm", "plain"}
    if "gemm" in only:
        # the fp32 SIMT GEMM form (64-walker tiles, register-blocked x'Px from shared memory)
        samp_gemm = graphs(sfs["gemm"].create_sampler(seed_base, WALKERS, dP))
        gemm_value, _, _ = timed_jobs(samp_gemm, max(1, min(args.steps, 2)), 1)
        samp_gemm.release()
    if "plain" in only:
        # the plain FP32 form (one thread per walker, the reference's kernel structure)
        samp_plain = graphs(sfs["plain"].create_sampler(seed_base, WALKERS, dP))
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
    peaks = measured_peaks()
    achieved = bytes_launch / t_launch / 1e9
    traffic = profile_traffic()

    # e2e: the same job through the C ABI from host buffers
    e2e_times = []
    h2d = P.nbytes
    d2h = 0
    for k in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s2 = graphs(sfs["tensor"].create_sampler(seed_base + 31 * k, WALKERS, P.reshape(-1)))
        res, mean, var, hist = job(s2, seed_base + 31 * k)
        s2.release()
        e2e_times.append(time.perf_counter() - t0)
        d2h = (8 + 3 * DIM * 8 + 2 * DIM * 8 + hist.limits.nbytes + hist.pdf.nbytes
               + hist.bin_ranks.nbytes)
    e2e_value = WALKERS * (BURN + RUN) * world / statistics.median(e2e_times)

    # the jobs' result: posterior means against the analytic mean 0.  Two standard
    # errors: acor's sigma of each job, and the spread of the run means over the
    # independent timed jobs (replicas with their own seeds), which needs no estimate of
    # the autocorrelation time.
    acs = [r[0]["autocorrelation"] for r in results if r[0]["autocorrelation"] is not None]
    res = results[-1][0]
    ac = res["autocorrelation"]
    result = {"acceptance_rate": res["acceptance_rate"], "dims": DIM, "jobs": len(results)}
    if ac is not None:
        tau = np.asarray(ac.tau, np.float64)
        result["tau_max"] = float(np.max(tau))
        result["means_within_3se_acor"] = int(np.sum(np.abs(ac.mean) <= 3 * ac.sigma))
        result["max_abs_mean_over_posterior_sd"] = float(
            np.max(np.abs(ac.mean) / np.sqrt(np.diag(sigma))))
    if len(acs) >= 3:
        m = np.array([a.mean for a in acs])                 # jobs x dims
        sd = m.std(axis=0, ddof=1)                          # s.e. of one job's mean
        grand = m.mean(axis=0)
        result["replica_se"] = {
            "jobs": len(acs),
            "job_means_within_3se": float(np.mean(np.abs(m) <= 3 * sd[None, :])),
            "grand_mean_within_3se_dims": int(np.sum(np.abs(grand) <= 3 * sd / np.sqrt(len(acs)))),
            "acor_sigma_over_replica_sd_median": float(
                np.nanmedian(np.nanmean([a.sigma for a in acs], axis=0) / sd))}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_sample(10.0)

    configs = None
    if rank == 0 and world == 1 and not args.no_configs:
        samp.release()
        samp = None
        for x in sfs.values():
            x.release()
        sfs = {}
        configs = measure_configs()

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
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": achieved / peaks["hbm_gbs"], "traffic": traffic,
                         "peak_kind": peaks["kind"],
                         "kernel": "bay_tcr_bare (GEMM form on the tensor cores, resident matrix)",
                         "launch_us": t_launch * 1e6,
                         "fp32_tflops": flop_launch / t_launch / 1e12},
            "cpu_baseline": cpu,
            "forms": {"tensor": value, "gemm_fp32_simt": gemm_value, "plain_fp32": plain_value,
                      "speedup_vs_plain": value / plain_value if plain_value else None},
            "logfn_err_vs_fp64": err,
            "autotune": tune,
            "clocks": clocks.summary(),
            "result": result,
        }
        if configs is not None:
            line["configs"] = configs
        if NO_GRAPHS:
            line["config"]["graphs"] = "off (--no-graphs: kernels launched one by one)"
        print(json.dumps(line))
    if samp is not None:
        samp.release()
    for x in sfs.values():
        x.release()
    f.release()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
