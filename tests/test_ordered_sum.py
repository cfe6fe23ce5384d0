"""The warp-step left-to-right FP64 sum (xb_ordered_sum_*) against the serial
loop of the reference's sigma-clip sums (bachUtil.cpp:34-128): equal bit for
bit on inputs built to hit every branch of the steps (binade crossings, exact
ties on the running sum's grid, zeros, subnormals, huge dynamic range,
negative terms and running sums, infinities)."""
import numpy as np
import pytest


def serial(c):
    s = 0.0
    for x in c:
        s += float(x)
    return s


def cases():
    rng = np.random.default_rng(20261204)
    out = []
    for n in (0, 1, 2, 31, 32, 33, 64, 100, 512, 1152):
        out.append(rng.uniform(0, 1e4, n))                          # chunk sums of pixels
        out.append(rng.uniform(0, 1e4, n) ** 2)                     # and of their squares
    for _ in range(40):
        n = int(rng.integers(1, 700))
        k = rng.integers(0, 1 << 22, n).astype(np.float64)
        out.append(k * 2.0 ** int(rng.integers(-30, 10)))          # few mantissa bits: ties
        out.append(np.exp(rng.uniform(-60, 60, n)))                 # dynamic range
        x = rng.uniform(0, 1, n)
        x[rng.uniform(0, 1, n) < 0.3] = 0.0                         # zeros
        out.append(x)
        out.append(rng.uniform(0.99, 1.01, n) * 2.0 ** int(rng.integers(0, 40)))  # near binades
    # every term a half-ulp of the running sum after the first
    # leading and inner runs of zeros (the substamp windows' skipped pixels),
    # with negative zeros among them
    z = np.zeros(441)
    z[180:200] = rng.uniform(1e3, 5e4, 20)
    z[250:260] = rng.uniform(1e3, 5e4, 10)
    out.append(z)
    out.append(np.concatenate([np.zeros(100), [-0.0, 0.0, -0.0, 3.5, -0.0, 1e-300]]))
    out.append(np.array([-0.0] * 70))
    out.append(np.array([1.0] + [2.0 ** -53] * 200))
    out.append(np.array([1.0] + [3 * 2.0 ** -53] * 200))
    out.append(np.array([2.0 ** 52] + [0.5, 1.5, 2.5, 0.5] * 50))
    # subnormal terms and sums
    out.append(np.array([5e-324] * 40 + [1e-310] * 40 + [1.0] * 10))
    # negatives (the serial branch) and a negative running sum
    out.append(np.array([1.0, -3.0, 2.0, 0.25, 1e-3, -1e-3] * 30))
    out.append(rng.normal(0, 1, 300))
    # infinities and the largest doubles
    out.append(np.array([1.0, 1e308, 1e308, 1.0]))
    out.append(np.array([1.0, np.inf, 1.0]))
    return out


def test_host_steps_equal_serial_loop():
    import xbach
    for i, c in enumerate(cases()):
        a, b = xbach.ordered_sum_host(c), serial(c)
        assert np.float64(a).tobytes() == np.float64(b).tobytes(), (i, len(c), a, b)


@pytest.mark.gpu
def test_warp_steps_equal_serial_loop():
    import ctypes
    import torch
    import xbach
    L = xbach.lib()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for i, c in enumerate(cases()):
        dc = torch.from_numpy(np.ascontiguousarray(c, dtype=np.float64)).cuda() if len(c) else out
        rc = L.xb_ordered_sum_device(ctypes.c_void_p(dc.data_ptr()), len(c),
                                     ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0
        torch.cuda.synchronize()
        a, b = float(out.cpu()[0]), serial(c)
        assert np.float64(a).tobytes() == np.float64(b).tobytes(), (i, len(c), a, b)


def float_cases():
    rng = np.random.default_rng(5)
    out = []
    for _ in range(60):
        n = int(rng.integers(1, 500))
        v = np.zeros(n, np.float32)
        on = rng.uniform(0, 1, n) < rng.uniform(0.05, 1.0)
        v[on] = np.exp(rng.uniform(-20, 11, on.sum()))               # pixels above sky
        out.append(v)
        out.append(rng.uniform(0, 6e4, n).astype(np.float32))
        out.append((rng.integers(0, 1 << 12, n) * 2.0 ** int(rng.integers(-30, 8))).astype(np.float32))
    out.append(np.array([-0.0, 0.0, -1.5, 2.0, -0.0, 1e-45, 3e38, 3e38], dtype=np.float32))
    out.append(np.array([1.0] + [2.0 ** -53] * 40, dtype=np.float32))  # half-ulp ties of the sum
    return out


@pytest.mark.gpu
def test_warp_steps_equal_serial_loop_f32():
    import ctypes
    import torch
    import xbach
    L = xbach.lib()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    for i, c in enumerate(float_cases()):
        dc = torch.from_numpy(c).cuda()
        rc = L.xb_ordered_sum_device_f32(ctypes.c_void_p(dc.data_ptr()), len(c),
                                         ctypes.c_void_p(out.data_ptr()), None)
        assert rc == 0
        torch.cuda.synchronize()
        a, b = float(out.cpu()[0]), serial(c.astype(np.float64))
        assert np.float64(a).tobytes() == np.float64(b).tobytes(), (i, len(c), a, b)

