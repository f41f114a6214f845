"""HDI utilities against the reference's util_test.clj fixtures (tests/golden/golden.json,
extracted by make_golden.py)."""
import numpy as np


def test_hdi_rank_count(golden):
    from bayadera_gb300 import util
    h = golden["hdi"]
    pdf = np.array(h["pdf"], np.float32)
    asum = float(np.sum(np.abs(pdf), dtype=np.float32))
    for c in h["rank_count"]:
        mass = c["mass"] / asum if c["scaled"] else c["mass"]
        assert util.hdi_rank_count(h["bin_rank"], pdf, mass) == c["want"], c


def test_hdi_bins(golden):
    from bayadera_gb300 import util
    h = golden["hdi"]
    for c in h["bins"]:
        assert util.hdi_bins(h["bin_rank"], c["cnt"]) == c["want"], c


def test_hdi_regions(golden):
    from bayadera_gb300 import util
    h = golden["hdi"]
    for c in h["regions"]:
        got = util.hdi_regions(h["limits"], h["bin_rank"], c["cnt"])
        want = np.array(c["want"]).reshape(c["cols"], 2).T
        assert got.shape == want.shape
        assert np.linalg.norm(got - want) <= c["tol"], (c, got)


def test_hdi_of_histogram(golden):
    from bayadera_gb300 import util
    from bayadera_gb300.engine import Histogram
    h = golden["hdi"]
    hist = Histogram(np.array(h["limits"])[:, None], np.array(h["pdf"])[:, None],
                     np.array(h["bin_rank"])[:, None])
    cnt = util.hdi_rank_count(h["bin_rank"], h["pdf"], 0.95)
    assert cnt == 71   # most of this fixture's mass is spread thinly over the tail bins
    np.testing.assert_allclose(util.hdi(hist, 0, 0.95),
                               util.hdi_regions(h["limits"], h["bin_rank"], cnt))
