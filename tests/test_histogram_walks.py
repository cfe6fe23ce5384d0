"""The histogram walks of the stamp statistics (createHistogram,
cl_kern/sss.cl:190-324; the oracle's restatement in oracle/xbach_oracle.cpp)
against the way k_stamp_stats forms them (csrc/xb_sss.cu, restated here in
Python): prefix sums C of the 256 bin counts, the sliding window of lower
index L ending at the first U in [L+1, 255] with C[U] - C[L] >= tenth, the
densest window chosen by exact integer cross products (first one on ties),
and the mode and quartile walks as binary searches on C.  The GPU parity
tests check the kernel itself; this checks the reformulation on histograms
built for its corner cases (empty bins, all pixels at either end, density
ties, one nonzero bin, counts from 1 to millions)."""
import math

import numpy as np


def serial(bins, ok):
    """The reference's walks in FP64, as the oracle runs them."""
    sum_bins, max_dens = 0.0, 0.0
    lo, up, max_index = 1, 1, -1
    while up < 255:
        while sum_bins < ok / 10.0 and up < 255:
            sum_bins += bins[up]
            up += 1
        if sum_bins / (up - lo) > max_dens:
            max_dens = sum_bins / (up - lo)
            max_index = lo
        sum_bins -= bins[lo]
        lo += 1
    if max_index < 0 or max_index > 255:
        max_index = 0
    sum_bins, sum_expect = 0.0, 0.0
    i = max_index
    while sum_bins < ok / 10.0 and i < 255:
        sum_bins += bins[i]
        sum_expect += i * bins[i]
        i += 1
    mode = sum_expect / sum_bins + 0.5 if sum_bins else math.nan
    lower, upper = ok * 0.25, ok * 0.75
    sum_bins, i = 0.0, 0
    while sum_bins < lower:
        sum_bins += bins[i]
        i += 1
    lower = i - (sum_bins - lower) / bins[i - 1]
    while sum_bins < upper:
        sum_bins += bins[i]
        i += 1
    upper = i - (sum_bins - upper) / bins[i - 1]
    return max_index, mode, lower, upper


def prefix(bins, ok):
    """The prefix-sum form of k_stamp_stats."""
    C = [0] * 257
    CE = [0] * 257
    for i in range(256):
        C[i + 1] = C[i] + int(bins[i])
        CE[i + 1] = CE[i] + i * int(bins[i])
    tenth = math.ceil(ok / 10.0)

    def first_at_least(lo, hi, target):
        while lo < hi:
            mid = (lo + hi) >> 1
            if C[mid] >= target:
                hi = mid
            else:
                lo = mid + 1
        return lo

    bN, bD, bL = 0, 1, -1
    for L in range(1, 255):
        if L > 1 and first_at_least(L, 255, C[L - 1] + tenth) >= 255:
            continue
        U = first_at_least(L + 1, 255, C[L] + tenth)
        S, D = C[U] - C[L], U - L
        if S * bD > bN * D:  # L increases: the first densest stays
            bN, bD, bL = S, D, L
    max_index = 0 if bL < 0 else bL
    i_end = first_at_least(max_index + 1, 255, C[max_index] + tenth)
    S, E = C[i_end] - C[max_index], CE[i_end] - CE[max_index]
    mode = float(E) / float(S) + 0.5 if S else math.nan
    lower, upper = ok * 0.25, ok * 0.75
    i1 = first_at_least(0, 256, math.ceil(lower))
    lower = i1 - (float(C[i1]) - lower) / bins[i1 - 1]
    i2 = first_at_least(i1, 256, math.ceil(upper))
    upper = i2 - (float(C[i2]) - upper) / bins[i2 - 1]
    return max_index, mode, lower, upper


def histograms():
    rng = np.random.default_rng(3)
    out = []
    for _ in range(400):
        kind = int(rng.integers(0, 6))
        b = np.zeros(256, np.int64)
        if kind == 0:   # a sky peak
            c = int(rng.integers(1, 255))
            w = float(rng.uniform(0.5, 40))
            n = int(rng.integers(1, 20000))
            idx = np.clip(np.round(rng.normal(c, w, n)).astype(int), 0, 255)
            np.add.at(b, idx, 1)
        elif kind == 1:  # sparse
            k = int(rng.integers(1, 6))
            b[rng.integers(0, 256, k)] = rng.integers(1, 50, k)
        elif kind == 2:  # everything at the ends
            b[0] = int(rng.integers(0, 100))
            b[255] = int(rng.integers(1, 100))
        elif kind == 3:  # flat: density ties everywhere
            b[1:255] = int(rng.integers(1, 5))
        elif kind == 4:  # large counts
            b[:] = rng.integers(0, 3_000_000, 256)
        else:            # random with holes
            b[:] = rng.integers(0, 4, 256) * (rng.uniform(0, 1, 256) < 0.3)
        if b.sum() == 0:
            b[int(rng.integers(0, 256))] = 1
        out.append(b)
    one = np.zeros(256, np.int64)
    one[100] = 7
    out.append(one)
    return out


def same(a, b):
    return (a == b) or (isinstance(a, float) and math.isnan(a) and math.isnan(b))


def test_prefix_walks_equal_serial_walks():
    for k, b in enumerate(histograms()):
        ok = int(b.sum())
        r_serial, r_prefix = serial(b, ok), prefix(b, ok)
        for x, y in zip(r_serial, r_prefix):
            assert same(x, y), (k, r_serial, r_prefix)
