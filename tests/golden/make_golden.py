"""Extract the reference's golden vectors for the stretch-move path into fixtures.

Reads the reference's own test file
  test/clojure/uncomplicate/bayadera/internal/nvidia_gtx_test.clj
and its acor series fixtures
  test/clojure/uncomplicate/bayadera/internal/acor-data-{67,367,112640}
and writes
  tests/golden/golden.json      -- every literal value asserted on the path
  tests/golden/acor_series.npz  -- the three acor series as float32

Run once in a checkout that has the reference tree:
  python tests/golden/make_golden.py /path/to/bayadera
The fixtures are committed; nothing reads the reference at test time.
"""
import json
import os
import re
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def _nums(s):
    return [float(t) for t in re.findall(r"-?\d+\.?\d*(?:E-?\d+)?", s)]


def _after(text, anchor, start=0):
    i = text.index(anchor, start)
    return i + len(anchor)


def _vector_after(text, anchor, start=0):
    """The first [...] or (list ...) literal after `anchor`."""
    i = _after(text, anchor, start)
    m = re.compile(r"=>\s*(\[[^\]]*\]|\(list[^)]*\)|\(map float \[[^\]]*\]\))").search(text, i)
    return _nums(m.group(1)), m.end()


def _scalar_after(text, anchor, start=0):
    i = _after(text, anchor, start)
    m = re.compile(r"=>\s*(\(roughly\s+[^)]*\)|\(float\s+[^)]*\)|-?\d+\.?\d*(?:E-?\d+)?)").search(text, i)
    return _nums(m.group(1)), m.end()


def extract(ref_root):
    tdir = os.path.join(ref_root, "test/clojure/uncomplicate/bayadera/internal")
    src = open(os.path.join(tdir, "nvidia_gtx_test.clj")).read()
    g = {"source": "test/clojure/uncomplicate/bayadera/internal/nvidia_gtx_test.clj"}

    # ---- direct samplers (nvidia_gtx_test.clj:38-107), seed 123, n = 10000
    samplers = {}
    for name, anchor in [("uniform", "direct sampler for Uniform"),
                         ("gaussian", "direct sampler for Gaussian"),
                         ("erlang", "direct sampler for Erlang"),
                         ("exponential", "direct sampler for Exponential")]:
        i = src.index(anchor)
        pm = re.compile(r"params \(vctr neanderthal-factory (\[[^\]]*\])\)").search(src, i)
        first, j = _vector_after(src, "(subvector sample-1d 0 4))", i)
        last, j = _vector_after(src, "(subvector sample-1d 9996 4))", j)
        mx, j = _scalar_after(src, "(imax sample-1d))", j)
        mn, j = _scalar_after(src, "(imin sample-1d))", j)
        mean, j = _scalar_after(src, "(mean sample-1d)", j)
        samplers[name] = {"params": _nums(pm.group(1)), "seed": 123, "n": 10000,
                          "first4": first, "last4": last, "max": mx[0], "min": mn[0],
                          "mean": mean[0]}
    g["direct_samplers"] = samplers

    # ---- stretch, uniform model (nvidia_gtx_test.clj:173-258)
    i = src.index('"Nvidia GTX stretch with Uniform model."')
    steps = []
    j = i
    for _ in range(4):
        v, j = _vector_after(src, "(take 4 (native (row (sample! uniform-sampler) 0)))", j)
        steps.append(v)
    relaunch = []
    for _ in range(2):
        v, j = _vector_after(src, "(take 4 (native (row res 0)))", j)
        relaunch.append(v)
    accu_first4, j = _vector_after(src, "(take 4 (native (row res 0)))", j)
    means_acc, j = _vector_after(src, "(seq means-acc-array)", j)
    accept, j = _vector_after(src, "(seq accept-array)", j)
    total, j = _scalar_after(src, "(sum acc)", j)
    g["stretch_uniform"] = {
        "wgs": 256, "walkers": 44 * 256, "seed": 123, "a": 2.0,
        "params": [-1.0, 2.0], "limits": [-1.0, 2.0],
        "sample_steps_first4": steps,
        "relaunch_first4": relaunch,
        "accu_first4": accu_first4,
        "accu_means_blocks_first10": means_acc,
        "accu_accept_blocks_first10": [int(x) for x in accept],
        "accu_means_total": total[0],
    }

    # ---- stretch, gaussian model (nvidia_gtx_test.clj:260-277)
    i = src.index('"Nvidia GTX stretch with Gaussian model."')
    j = i
    gs = []
    for _ in range(3):
        v, j = _vector_after(src, "(take 4 (native (row (sample! gaussian-sampler) 0)))", j)
        gs.append(v)
    g["stretch_gaussian"] = {"wgs": 256, "walkers": 44 * 256, "seed": 123, "a": 2.0,
                             "params": [3.0, 1.0], "limits": [-7.0, 7.0],
                             "sample_steps_first4": gs}

    # ---- burn-in, gaussian model (nvidia_gtx_test.clj:279-296)
    i = src.index('"Nvidia GTX stretch burn-in with Gaussian model."')
    mean, j = _scalar_after(src, "(first (native! (mean (sample! gaussian-sampler))))", i)
    nth, j = _vector_after(src, "(take-nth 1500 (native! (row (sample! gaussian-sampler) 0)))", j)
    sd, j = _scalar_after(src, "(first (native! (sd (sample! gaussian-sampler))))", j)
    g["burn_in_gaussian"] = {"wgs": 256, "walkers": 44 * 256, "init_seed": 123, "seed": 124,
                             "steps": 100, "a": 1.5, "params": [3.0, 1.0], "limits": [-7.0, 7.0],
                             "mean": mean[0], "take_nth_1500": nth, "sd": sd[0]}

    # ---- engine statistics (nvidia_gtx_test.clj:298-318)
    i = src.index('"Test MCMC stretch engine."')
    acc, j = _scalar_after(src, "(acc-rate! engine a)", i)
    tau, j = _scalar_after(src, "(run-sampler! engine 63670 a))) 0)", j)
    g["engine_gaussian"] = {"wgs": 256, "walkers": 2 * 44 * 256, "seed": 123, "a": 8.0,
                            "params": [200.0, 1.0], "limits": [180.0, 220.0],
                            "burn_in": 5120, "acc_rate": acc[0], "acc_rate_tol": acc[1],
                            "run_steps": 63670, "tau": tau[0], "tau_tol": tau[1]}

    # ---- acor (nvidia_gtx_test.clj:320-358)
    i = src.index('"Test MCMC acor."')
    t67, j = _vector_after(src, "(seq (:tau autocorrelation))", i)
    s67, j = _scalar_after(src, "(entry (:sigma autocorrelation) 0)", j)
    t367, j = _vector_after(src, "(seq (:tau autocorrelation))", j)
    s367, j = _scalar_after(src, "(entry (:sigma autocorrelation) 0)", j)
    tbig, j = _scalar_after(src, "(second (:tau autocorrelation))", j)
    sbig, j = _scalar_after(src, "(entry (:sigma autocorrelation) 0)", j)
    g["acor"] = {
        "wgs": 256,
        "67": {"row1": "times 2", "tau": t67, "sigma0": s67[0]},
        "367": {"row1": "plus 1", "tau": t367, "sigma0": s367[0]},
        "112640": {"row1": "times 2", "tau1": tbig[0], "tau1_tol": tbig[1],
                   "sigma0": sbig[0], "sigma0_tol": sbig[1]},
    }

    # ---- posterior engine, beta-binomial model (nvidia_gtx_test.clj:133-159): n, z, a, b,
    # the points (range 0.001 1 0.001) as a 1 x 200 matrix, the constant that separates the
    # posterior's log density from the conjugate beta's, and the binomial evidence
    i = src.index('"Nvidia GTX posterior engine with Beta-Binomial model."')
    nz = {k: float(re.compile(r"\b%s (\d+)" % k).search(src, i).group(1)) for k in ("n", "z", "a", "b")}
    pm = re.compile(r"\(ge neanderthal-factory 1 (\d+) \(range ([\d.]+) ([\d.]+) ([\d.]+)\)\)").search(src, i)
    const = re.compile(r"x-beta-log-pdf\) (-?[\d.]+)\)\) => \(roughly 0\.0 ([\d.]+)\)").search(src, i)
    ev = re.compile(r"\(evidence binomial-lik-engine lik-params x\) => (-?[\d.]+E-?\d+)").search(src, i)
    g["beta_binomial"] = {"n": nz["n"], "z": nz["z"], "a": nz["a"], "b": nz["b"],
                          "points": int(pm.group(1)), "start": float(pm.group(2)),
                          "step": float(pm.group(4)),
                          "log_ratio": float(const.group(1)), "log_ratio_tol": float(const.group(2)),
                          "evidence": float(ev.group(1))}

    # ---- HDI utilities (test/clojure/uncomplicate/bayadera/util_test.clj): the fixture
    # pdf / bin ranks / limits and the asserted hdi-rank-count, hdi-bins, hdi-regions
    usrc = open(os.path.join(ref_root, "test/clojure/uncomplicate/bayadera/util_test.clj")).read()
    lims = [float(x) for x in re.search(r"l (\d+)\s+u (\d+)", usrc).groups()]
    pdf = _nums(re.search(r"tpdf \(fv \[([^\]]*)\]\)", usrc).group(1))
    rm = re.search(r"tbin-rank \(fv \(op \[([^\]]*)\] \(range (\d+) (\d+)\)\)\)", usrc)
    rank = _nums(rm.group(1)) + [float(v) for v in range(int(rm.group(2)), int(rm.group(3)))]
    counts = []
    for m in re.finditer(r"\(hdi-rank-count (\(/ )?([\d.]+)( tpdf-asum\))? tbin-rank tpdf\) => (\d+)",
                         usrc):
        counts.append({"mass": float(m.group(2)), "scaled": bool(m.group(1)),
                       "want": int(m.group(4))})
    bins = [{"cnt": int(m.group(1)), "want": _nums(m.group(2))}
            for m in re.finditer(r"\(hdi-bins tbin-rank (\d+)\) => \[([^\]]*)\]", usrc)]
    regions = [{"cnt": int(m.group(1)), "cols": int(m.group(2)), "want": _nums(m.group(3)),
                "tol": float(m.group(4))}
               for m in re.finditer(r"\(hdi-regions tlimits tbin-rank (\d+)\) \(fge 2 (\d+) \[([^\]]*)\]\)\)\) "
                                    r"=> \(roughly 0 ([\d.]+)\)", usrc)]
    g["hdi"] = {"source": "test/clojure/uncomplicate/bayadera/util_test.clj", "limits": lims,
                "pdf": pdf, "bin_rank": rank, "rank_count": counts, "bins": bins,
                "regions": regions}

    series = {}
    for n in (67, 367, 112640):
        with open(os.path.join(tdir, "acor-data-%d" % n)) as f:
            series["n%d" % n] = np.array([float(x) for x in f.read().split()], dtype=np.float32)
    return g, series


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path of the uncomplicate/bayadera source tree>")
    g, series = extract(sys.argv[1])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(g, f, indent=1)
    np.savez_compressed(os.path.join(HERE, "acor_series.npz"), **series)
    print("wrote golden.json and acor_series.npz")


if __name__ == "__main__":
    main()
