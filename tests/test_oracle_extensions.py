"""The oracle's restatement of the HOTPANTS-style extensions (xb_params gain,
readNoise, convPerPixel), checked through properties the mathematics fixes:

* without read noise the chi^2 denominator is (|t| + |s|) / gain, so every
  stamp chi^2 scales by exactly `gain` (a power of two keeps it exact) while
  every decision, being scale-free (sigma clipping of the chi^2 set, the
  ratio of the two directions' merits), stays the same;
* with a spatially constant kernel (kernel order 0) the per-pixel kernel is
  the per-block kernel, so both convolutions agree to rounding;
* with an unbounded gain and read noise 0.5 every fit weight is exactly 2, so
  the weighted normal equations are exactly twice the unweighted ones and
  every decision, the solution and the images are bit-identical."""
import numpy as np


def _run(oracle, test01, **kw):
    ref = oracle.run(oracle.default_params(**kw), test01["T"], test01["S"])
    assert ref.status == 0
    return ref


def test_gain_scales_every_stamp_chi2(oracle, test01, test01_oracle):
    base = test01_oracle
    g2 = _run(oracle, test01, gain=2.0)
    assert np.array_equal(g2.array("solution", np.float64), base.array("solution", np.float64))
    assert np.array_equal(g2.array("ksc_rejects", np.int32), base.array("ksc_rejects", np.int32))
    a, b = g2.array("ksc_sig_last", np.float64), base.array("ksc_sig_last", np.float64)
    valid = b != -1.0
    assert valid.any() and np.array_equal(a[valid], 2.0 * b[valid]) and np.all(a[~valid] == -1.0)
    assert np.array_equal(g2.array("diff", np.float64), base.array("diff", np.float64))


def test_per_pixel_kernel_equals_block_kernel_when_constant(oracle, test01):
    blk = _run(oracle, test01, kernelOrder=0)
    pp = _run(oracle, test01, kernelOrder=0, convPerPixel=1)
    assert np.array_equal(pp.array("solution", np.float64), blk.array("solution", np.float64))
    assert np.array_equal(pp.array("mask", np.uint16), blk.array("mask", np.uint16))
    for k in ("conv", "diff"):
        a, b = pp.array(k, np.float64), blk.array(k, np.float64)
        scale = np.abs(blk.array("conv", np.float64)).max()
        assert np.abs(a - b).max() <= 1e-12 * scale, k


def test_per_pixel_kernel_is_the_polynomial_kernel_at_each_pixel(oracle, test01, test01_oracle):
    """Kernel order 2: each interior pixel equals the direct sum of the kernel
    evaluated at that pixel (basis coefficients from the solution, cd.cl
    makeKernelCoeffs order) times the flipped window, plus the background,
    normalised as conv.cl does; and the images differ from the per-block
    ones (test01's fit varies strongly across the frame)."""
    pp = _run(oracle, test01, convPerPixel=1)
    sol = pp.array("solution", np.float64)
    fK, hK, kO = 21, 10, 2
    n_psf, n_c2 = 49, 6
    vec = pp.array("basis", np.float64)[:n_psf * fK * fK].reshape(n_psf, fK, fK)
    T, S = test01["T"], test01["S"]
    h, w = T.shape
    conv_t = pp.scalar("convTemplate") == 1
    I = T if conv_t else S
    scale = 1.0 / pp.scalar("kernSum") if conv_t else 1.0  # normalizeTemplate = 1
    conv = pp.array("conv", np.float64).reshape(h, w)

    def mono(xf, yf, order):
        return [xf ** i * yf ** j for i in range(order + 1) for j in range(order + 1 - i)]

    for x, y in [(hK, hK), (50, 60), (165, 165), (300, 40), (w - hK - 1, h - hK - 1)]:
        xf, yf = (x - 0.5 * w) / (0.5 * w), (y - 0.5 * h) / (0.5 * h)
        P = mono(xf, yf, kO)
        c = [sol[1]] + [sum(sol[2 + (n - 1) * n_c2 + t] * P[t] for t in range(n_c2))
                        for n in range(1, n_psf)]
        kern = np.tensordot(np.array(c), vec, axes=1)
        win = I[y - hK:y + hK + 1, x - hK:x + hK + 1]
        bg = sum(sol[(n_psf - 1) * n_c2 + 2 + t] * m for t, m in enumerate(mono(xf, yf, 1)))
        want = ((kern[::-1, ::-1] * win).sum() + bg) * scale
        assert abs(conv[y, x] - want) <= 1e-11 * np.abs(conv).max(), (x, y, conv[y, x], want)
    assert not np.array_equal(pp.array("conv", np.float64), test01_oracle.array("conv", np.float64))


def test_weighted_fit_with_constant_weight_two_is_exact(oracle, test01):
    kw = dict(gain=1e300, readNoise=0.5)
    plain = _run(oracle, test01, **kw)
    wfit = _run(oracle, test01, fitWeighted=1, **kw)
    for k in ("solution", "ksc_sig_last", "conv", "diff"):
        assert np.array_equal(wfit.array(k, np.float64), plain.array(k, np.float64)), k
    for k in ("ksc_rejects", "cur"):
        assert np.array_equal(wfit.array(k, np.int32), plain.array(k, np.int32)), k
    assert np.array_equal(2.0 * plain.array("ksc_matrix0", np.float64),
                          wfit.array("ksc_matrix0", np.float64))


def test_weighted_fit_changes_the_solution(oracle, test01, test01_oracle):
    """Poisson weights (gain 1, read noise 5): another solution of the same
    system shape, with every stage completing."""
    w = _run(oracle, test01, fitWeighted=1, readNoise=5.0)
    a, b = w.array("solution", np.float64), test01_oracle.array("solution", np.float64)
    assert a.shape == b.shape and np.all(np.isfinite(a)) and not np.array_equal(a, b)


def test_oracle_input_mask_excludes_pixels(oracle, test01, test01_oracle):
    """The oracle's input mask: the pixels get INPUT_MASK | BAD_INPUT at
    init, end BAD_OUTPUT with the bad-output value, and an empty mask gives
    the unmasked run bit for bit."""
    INPUT_MASK, BAD_INPUT, BAD_OUTPUT = 1 << 5, 1 << 7, 1 << 12
    T, S = test01["T"], test01["S"]
    m = np.zeros(T.shape, np.uint8)
    m[100:110, 150:170] = 1
    m[200, :] = 1
    r = oracle.run(oracle.default_params(), T, S, mask=m)
    assert r.status == 0
    init = r.array("mask_init", np.uint16).reshape(T.shape)
    assert np.all((init[m != 0] & (INPUT_MASK | BAD_INPUT)) == INPUT_MASK | BAD_INPUT)
    fin = r.array("mask", np.uint16).reshape(T.shape)
    assert np.all(fin[m != 0] & BAD_OUTPUT)
    assert np.all(r.array("diff", np.float64).reshape(T.shape)[m != 0] == 1e-30)
    empty = oracle.run(oracle.default_params(), T, S, mask=np.zeros_like(m))
    for k in ("solution", "diff", "mask"):
        dt = np.uint16 if k == "mask" else np.float64
        assert np.array_equal(empty.array(k, dt), test01_oracle.array(k, dt)), k
