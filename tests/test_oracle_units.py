"""Known-answer checks of the oracle's building blocks."""
import ctypes

import numpy as np


def _clip(oracle, data, it=3, alpha=3.0):
    m, s = ctypes.c_double(), ctypes.c_double()
    d = np.ascontiguousarray(data, np.float64)
    oracle.lib.xbo_sigma_clip(d.ctypes.data, len(d), it, alpha,
                              ctypes.byref(m), ctypes.byref(s))
    return m.value, s.value


def test_sigma_clip_matches_direct_formula(oracle):
    rng = np.random.default_rng(7)
    d = rng.normal(100.0, 5.0, 5000)
    d[:20] = 1e4  # outliers
    keep = np.ones(len(d), bool)
    mean = sd = None
    prev, curr = len(d), 0
    for _ in range(3):
        if curr == prev:
            break
        curr = prev
        x = d[keep]
        mean = x.sum() / len(x)
        sd = np.sqrt((np.sum(x * x) - len(x) * mean * mean) / (len(x) - 1))
        clip = keep & (np.abs(d - mean) / sd > 3.0)
        keep &= ~clip
        prev = curr - clip.sum()
    m, s = _clip(oracle, d)
    assert abs(m - mean) < 1e-9 and abs(s - sd) < 1e-9


def test_sigma_clip_degenerate_inputs(oracle):
    # src/bachUtil.cpp:37-42 and :81-87: empty or single-point input
    assert _clip(oracle, np.zeros(0)) == (0.0, 1e10)
    assert _clip(oracle, np.array([5.0])) == (0.0, 1e10)


def test_ran1_range_and_determinism(oracle):
    a = np.empty(1000)
    b = np.empty(1000)
    oracle.lib.xbo_ran1_seq(-666, 1000, a.ctypes.data)
    oracle.lib.xbo_ran1_seq(-666, 1000, b.ctypes.data)
    assert np.array_equal(a, b)
    assert a.min() > 0.0 and a.max() < 1.0
    assert abs(a.mean() - 0.5) < 0.05


def test_lu_solve_matches_numpy(oracle):
    rng = np.random.default_rng(3)
    n = 40
    A = rng.normal(size=(n, n)) + n * np.eye(n)
    b = rng.normal(size=n)
    a1 = np.zeros((n + 1, n + 1))
    a1[1:, 1:] = A
    r1 = np.zeros(n + 1)
    r1[1:] = b
    rc = oracle.lib.xbo_lu_solve(a1.ctypes.data, n, r1.ctypes.data)
    assert rc == 0
    assert np.allclose(r1[1:], np.linalg.solve(A, b), rtol=1e-10, atol=1e-12)


def test_lu_zero_row_reports_error(oracle):
    n = 4
    a1 = np.zeros((n + 1, n + 1))
    a1[1:, 1:] = np.eye(n)
    a1[3, :] = 0.0
    r1 = np.ones(n + 1)
    assert oracle.lib.xbo_lu_solve(a1.ctypes.data, n, r1.ctypes.data) == 1
