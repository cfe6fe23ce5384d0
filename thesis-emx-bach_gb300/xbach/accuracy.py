"""Error figures of one difference-imaging result against another.

A run is compared either with the plain GPU path (the acceptance test of the
mixed path) or with the FP64 oracle.  The figures:

* difference pixels in units of the per-pixel noise,
  sigma_pix = sqrt(|target| + |conv| + 2 sigma_rn^2) (gain 1; target is the
  image the convolved one is subtracted from), over pixels neither run set to
  the 1e-30 border/bad value (in FP64 or FP32);
* kernel coefficients sol[1 .. nComp+1] and background terms
  sol[nComp+2 .. nComp+1+nBG] (the solution layout of the reference's
  fitKernel, cdkscUtil.cpp:585-684), as max |delta| / max |reference|;
* the photometric scale (kernel sum), relative.
"""
import numpy as np

SIGMA_RN = 5.0  # read noise of the synthetic frames, ADU


def layout(params):
    """(nComp, nBG) of a parameter set (xb_params or the oracle's)."""
    n_psf = sum((params.dg[i] + 1) * (params.dg[i] + 2) // 2 for i in range(params.nGauss))
    n_c2 = (params.kernelOrder + 1) * (params.kernelOrder + 2) // 2
    n_bg = (params.backgroundOrder + 1) * (params.backgroundOrder + 2) // 2
    return (n_psf - 1) * n_c2, n_bg


BAD_VALUES = (1e-30, float(np.float32(1e-30)))  # the bad-pixel value, FP64 and FP32


def is_bad(img):
    """Pixels holding the border / bad-output value 1e-30 (FP64 or FP32)."""
    img = np.asarray(img, dtype=np.float64)
    return (img == BAD_VALUES[0]) | (img == BAD_VALUES[1])


def diff_error(diff, diff_ref, conv_ref, target, sigma_rn=SIGMA_RN):
    diff = np.asarray(diff, dtype=np.float64)
    diff_ref = np.asarray(diff_ref, dtype=np.float64)
    ok = ~is_bad(diff) & ~is_bad(diff_ref)
    sigma = np.sqrt(np.abs(np.asarray(target, np.float64)) +
                    np.abs(np.asarray(conv_ref, np.float64)) + 2 * sigma_rn ** 2)
    e = np.abs(diff - diff_ref)[ok] / sigma[ok]
    if e.size == 0:
        return {"max_sigma": None, "rms_sigma": None, "pixels": 0}
    return {"max_sigma": float(e.max()), "rms_sigma": float(np.sqrt(np.mean(e * e))),
            "pixels": int(ok.sum())}


def _rel(a, r):
    den = float(np.max(np.abs(r))) if r.size else 0.0
    return float(np.max(np.abs(a - r)) / den) if den > 0 else float(np.max(np.abs(a - r)))


def fit_error(sol, sol_ref, n_comp, n_bg):
    sol = np.asarray(sol, np.float64)
    sol_ref = np.asarray(sol_ref, np.float64)
    k = slice(1, n_comp + 2)
    b = slice(n_comp + 2, n_comp + 2 + n_bg)
    return {"kernel_coeff_max_rel": _rel(sol[k], sol_ref[k]),
            "background_max_rel": _rel(sol[b], sol_ref[b]),
            "background_max_abs": float(np.max(np.abs(sol[b] - sol_ref[b])))}


def compare(run, ref, T, S, n_comp, n_bg, sigma_rn=SIGMA_RN):
    """run/ref: dicts with keys diff, conv, solution, kernSum, convTemplate."""
    target = S if ref["convTemplate"] else T
    out = {"same_direction": bool(run["convTemplate"] == ref["convTemplate"]),
           "kernel_sum_rel": float(abs(run["kernSum"] / ref["kernSum"] - 1.0))}
    out.update(fit_error(run["solution"], ref["solution"], n_comp, n_bg))
    out["diff"] = diff_error(run["diff"], ref["diff"], ref["conv"], target, sigma_rn)
    return out


def residual_noise(runs, T, S, sigma_rn=SIGMA_RN):
    """Fit quality of difference images without a ground truth: diff in
    units of sigma_pix (above), over the pixels every run kept.  A perfect
    kernel leaves noise; a poorer one leaves residuals around the stars,
    which widen the bulk of the distribution (robust_sigma = 1.4826 x the
    median absolute deviation, 1 for pure noise; p90 of |diff|/sigma).  The
    rms is dominated by cosmic rays, variable stars and defects, which no
    kernel removes.  runs: dicts with diff, conv, convTemplate."""
    ok = np.ones(np.shape(T), bool)
    for r in runs:
        ok &= ~is_bad(r["diff"])
    out = []
    for r in runs:
        target = S if r["convTemplate"] else T
        sigma = np.sqrt(np.abs(np.asarray(target, np.float64)) +
                        np.abs(np.asarray(r["conv"], np.float64)) + 2 * sigma_rn ** 2)
        e = np.asarray(r["diff"], np.float64)[ok] / sigma[ok]
        med = np.median(e)
        a = np.abs(e)
        out.append({"robust_sigma": float(1.4826 * np.median(np.abs(e - med))),
                    "p90_sigma": float(np.quantile(a, 0.9)),
                    "rms_sigma": float(np.sqrt(np.mean(e * e))), "pixels": int(ok.sum())})
    return out
