"""Host utilities on histograms (uncomplicate/bayadera/util.clj): the bin mapper and the
highest-density-interval (HDI) regions computed from a histogram's pdf and its bin ranks
(the bins in decreasing order of mass, as the histogram kernels return them)."""
import numpy as np


def bin_mapper(bin_count, lower, upper, offset=0.5):
    """bin-mapper (util.clj:40-49): bin index -> the point at `offset` within the bin."""
    width = (upper - lower) / bin_count
    return lambda i: lower + width * (i + offset)


def hdi_rank_count(bin_rank, pdf, mass=0.95):
    """hdi-rank-count (util.clj:51-65): the fewest top-ranked bins whose pdf mass reaches
    `mass` of the total (the total summed in float32, the masses added in double)."""
    pdf = np.asarray(pdf, np.float32)
    density = mass * float(np.sum(np.abs(pdf), dtype=np.float32))
    acc, i, n = 0.0, 0, len(bin_rank)
    while i < n and acc < density:
        acc += float(pdf[int(bin_rank[i])])
        i += 1
    return i


def hdi_bins(bin_rank, hdi_cnt):
    """hdi-bins (util.clj:67-83): the first hdi_cnt ranked bins grouped into contiguous
    regions, [start0, end0, start1, end1, ...]; bins more than one apart start a region."""
    v = sorted(float(b) for b in np.asarray(bin_rank)[:hdi_cnt])
    regions = [v[0]]
    last = v[0]
    for b in v[1:]:
        if b - last > 1.5:
            regions += [last, b]
        last = b
    regions.append(v[-1])
    return regions


def hdi_regions(limits, bin_rank, hdi_cnt):
    """hdi-regions (util.clj:85-99): a 2 x regions array of [lower, upper] bounds."""
    lower, upper = float(limits[0]), float(limits[1])
    width = (upper - lower) / len(bin_rank)
    b = hdi_bins(bin_rank, hdi_cnt)
    cnt = len(b) // 2
    out = np.zeros((2, cnt))
    for i in range(cnt):
        out[0, i] = lower + width * b[2 * i]
        out[1, i] = lower + width * (b[2 * i + 1] + 1.0)
    return out


def hdi(histogram, index, mass=0.95):
    """hdi (util.clj:101-110): the HDI regions holding `mass` of variable `index` of a
    Histogram(limits 2 x dim, pdf bins x dim, bin_ranks bins x dim)."""
    limits = np.asarray(histogram.limits)[:, index]
    ranks = np.asarray(histogram.bin_ranks)[:, index]
    pdf = np.asarray(histogram.pdf)[:, index]
    return hdi_regions(limits, ranks, hdi_rank_count(ranks, pdf, mass))
