"""Seeded synthetic template/science frame pairs.

Stand-ins for the survey frames the reference measures on (they are not
available): point sources with pixel-integrated Gaussian PSFs on a Poisson
sky with Gaussian read noise.  The science frame is the template scene scaled
by `scale`, seen through a broader PSF, plus a linear background, with a few
variable sources.  Optional cosmic-ray hits and clipped saturated stars.
Counter-based RNG (Philox) seeded per configuration, so a (config, frame)
pair is reproducible on any machine with the same numpy.
"""
import numpy as np
from scipy.special import erf

CONFIGS = {
    # 512x512, 1500 sources, FWHM 2.5 (template) / 3.5 (science)
    1: dict(size=512, n_src=1500, fwhm_t=(2.5, 2.5), fwhm_s=(3.5, 3.5),
            flux=(1e3, 1e6), cr_frac=0.0, n_sat=0, stamps=10,
            saturation=None),
    # 2048x2048, 20k sources, FWHM varying across the field, 1% cosmic-ray
    # pixels, 40 saturated stars; the detector saturates at 6e4 (every pixel
    # is clipped there and threshHigh sits at that level), 16x16 stamps
    2: dict(size=2048, n_src=20000, fwhm_t=(2.2, 3.2), fwhm_s=(3.0, 4.2),
            flux=(1e3, 1e6), cr_frac=0.01, n_sat=40, stamps=16,
            saturation=6e4),
    # 3072x3072 crowded field, 80k sources down to 1e2 ADU, FWHM varying
    # across the field, 20x20 stamps; fitted with 4 Gaussians (sigma
    # 0.6/1.2/2.4/4.8, degrees 6/4/3/2 -> 59 functions), kernel order 3,
    # background order 2 (see PARAMS_3)
    3: dict(size=3072, n_src=80000, fwhm_t=(2.2, 3.2), fwhm_s=(3.0, 4.2),
            flux=(1e2, 1e6), cr_frac=0.0, n_sat=0, stamps=20,
            saturation=None),
}

# Ranker field, preset 5: preset 2 at 4096^2 with 120k sources and 20x20
# stamps, plus defects on the substamps the fit would try first: in 2 % of
# the stamps a hot column of the science image (+300..3000 ADU over the
# stamp's rows) passes within 3 px of the stamp's brightest unsaturated star,
# in 5 % that star gets a variable companion 1.5-3 px away (flux 0.3-1 of the
# primary, science flux off by 20-40 %).
CONFIGS[5] = dict(CONFIGS[2], size=4096, n_src=120000, stamps=20, bad_col_frac=0.02,
                  binary_frac=0.05, chunk=16384)

# Basis and orders of preset 3 (keyword arguments of xbach.default_params).
PARAMS_3 = dict(nGauss=4, dg=[6, 4, 3, 2],
                bg=[1 / (2 * 0.6 ** 2), 1 / (2 * 1.2 ** 2), 1 / (2 * 2.4 ** 2), 1 / (2 * 4.8 ** 2)],
                kernelOrder=3, backgroundOrder=2)


def _render(img, xs, ys, fluxes, sigmas, chunk=None, r=None):
    """Adds pixel-integrated Gaussians (one sigma per source) into img.

    chunk: sources per pass (bounds the temporary arrays); every pass uses
    the radius of the widest source, so the image does not depend on it."""
    if len(xs) == 0:
        return
    if r is None:
        r = int(np.ceil(4.0 * sigmas.max())) + 1
    if chunk and len(xs) > chunk:
        for i in range(0, len(xs), chunk):
            _render(img, xs[i:i + chunk], ys[i:i + chunk], fluxes[i:i + chunk],
                    sigmas[i:i + chunk], None, r)
        return
    h, w = img.shape
    off = np.arange(-r, r + 1)
    cx = np.floor(xs).astype(np.int64)
    cy = np.floor(ys).astype(np.int64)
    px = cx[:, None] + off[None, :]                      # (n, k)
    py = cy[:, None] + off[None, :]
    s2 = (sigmas * np.sqrt(2.0))[:, None]
    gx = 0.5 * (erf((px + 0.5 - xs[:, None]) / s2) - erf((px - 0.5 - xs[:, None]) / s2))
    gy = 0.5 * (erf((py + 0.5 - ys[:, None]) / s2) - erf((py - 0.5 - ys[:, None]) / s2))
    vals = fluxes[:, None, None] * gy[:, :, None] * gx[:, None, :]   # (n, ky, kx)
    X = np.broadcast_to(px[:, None, :], vals.shape)
    Y = np.broadcast_to(py[:, :, None], vals.shape)
    ok = (X >= 0) & (X < w) & (Y >= 0) & (Y < h)
    idx = (Y[ok] * w + X[ok]).astype(np.int64)
    img += np.bincount(idx, weights=vals[ok], minlength=h * w).reshape(h, w)


def make_pair(config=1, frame=0, size=None, n_src=None, dtype=np.float32, **over):
    """Returns (template, science, info) for field preset `config` (see CONFIGS).

    frame: index of the pair within a batch (changes the seed).
    """
    cfg = dict(CONFIGS[config])
    if size is not None:
        cfg["size"] = size
    if n_src is not None:
        cfg["n_src"] = n_src
    seed = over.pop("seed", config)
    cfg.update(over)
    rng = np.random.Generator(np.random.Philox(key=seed * 1000003 + frame))
    n = cfg["size"]
    sky, rn, scale = 1000.0, 5.0, 1.1
    ns = cfg["n_src"]
    xs = rng.uniform(0, n - 1, ns)
    ys = rng.uniform(0, n - 1, ns)
    lf = np.log10(cfg["flux"])
    flux = 10.0 ** rng.uniform(lf[0], lf[1], ns)
    sat = np.zeros(ns, bool)
    if cfg["n_sat"]:
        k = rng.choice(ns, cfg["n_sat"], replace=False)
        flux[k] = 10.0 ** rng.uniform(6.5, 7.5, cfg["n_sat"])
        sat[k] = True
    var = rng.choice(ns, min(15, ns), replace=False)
    flux_s = flux * scale
    flux_s[var] *= 1.0 + rng.uniform(-0.2, 0.2, len(var))
    # defects on the brightest unsaturated star of chosen stamp cells
    bad_cols, binaries = [], []
    if cfg.get("bad_col_frac") or cfg.get("binary_frac"):
        g = cfg["stamps"]
        cell = np.minimum((xs * g / n).astype(int), g - 1) + g * np.minimum((ys * g / n).astype(int), g - 1)
        usable = (flux < 3e5) & ~sat
        add_x, add_y, add_f, add_fs = [], [], [], []
        for c in range(g * g):
            want_col = rng.random() < cfg.get("bad_col_frac", 0.0)
            want_bin = rng.random() < cfg.get("binary_frac", 0.0)
            if not (want_col or want_bin):
                continue
            idx = np.flatnonzero((cell == c) & usable)
            if len(idx) == 0:
                continue
            k = idx[np.argmax(flux[idx])]
            if want_bin:
                r, a = rng.uniform(1.5, 3.0), rng.uniform(0, 2 * np.pi)
                f2 = flux[k] * rng.uniform(0.3, 1.0)
                add_x.append(xs[k] + r * np.cos(a))
                add_y.append(ys[k] + r * np.sin(a))
                add_f.append(f2)
                add_fs.append(f2 * scale * (1.0 + rng.choice([-1, 1]) * rng.uniform(0.2, 0.4)))
                binaries.append((float(xs[k]), float(ys[k])))
            if want_col:
                x0 = int(np.clip(round(xs[k]) + rng.integers(-3, 4), 0, n - 1))
                cy0, cy1 = (c // g) * n // g, ((c // g) + 1) * n // g
                bad_cols.append((x0, cy0, cy1, float(rng.uniform(300.0, 3000.0))))
        if add_x:
            xs = np.concatenate([xs, np.clip(add_x, 0, n - 1)])
            ys = np.concatenate([ys, np.clip(add_y, 0, n - 1)])
            flux = np.concatenate([flux, add_f])
            flux_s = np.concatenate([flux_s, add_fs])

    def fwhm_at(rng_fwhm):
        a, b = rng_fwhm
        return a + (b - a) * xs / max(n - 1, 1)

    c = 1.0 / (2.0 * np.sqrt(2.0 * np.log(2.0)))
    sig_t = fwhm_at(cfg["fwhm_t"]) * c
    sig_s = fwhm_at(cfg["fwhm_s"]) * c
    T = np.zeros((n, n))
    S = np.zeros((n, n))
    _render(T, xs, ys, flux, sig_t, cfg.get("chunk"))
    _render(S, xs, ys, flux_s, sig_s, cfg.get("chunk"))
    xx = np.arange(n)[None, :].repeat(n, 0)
    S += 50.0 + 0.01 * xx
    T = rng.poisson(T + sky).astype(np.float64) + rng.normal(0.0, rn, T.shape)
    S = rng.poisson(S + sky).astype(np.float64) + rng.normal(0.0, rn, S.shape)
    if cfg["cr_frac"] > 0:
        for img in (T, S):
            m = rng.random(img.shape) < cfg["cr_frac"]
            img[m] += rng.uniform(5e3, 5e4, int(m.sum()))
    for x0, y0, y1, off in bad_cols:
        S[y0:y1, x0] += off
    if cfg["saturation"]:
        np.minimum(T, cfg["saturation"], out=T)
        np.minimum(S, cfg["saturation"], out=S)
    info = dict(config=config, frame=frame, stamps=cfg["stamps"], size=n, n_src=ns,
                threshHigh=cfg["saturation"] or 25000.0, bad_cols=bad_cols, binaries=binaries)
    return T.astype(dtype), S.astype(dtype), info


# Batched preset 4: pairs whose size, stamp grid, source density and
# science/template FWHM ratio are drawn from the frame's seed; otherwise
# preset 2 (FWHM 2.2-3.2 px across the template field, 1 % cosmic-ray
# pixels, 40 saturated stars, saturation 6e4).
SIZES_4 = (512, 1024, 2048, 3072, 4096)


def config4_draw(frame):
    """Size, stamp grid, density (sources per px^2) and FWHM ratio of pair
    `frame` of preset 4."""
    rng = np.random.Generator(np.random.Philox(key=4 * 1000003 + 104729 * (frame + 1)))
    size = int(SIZES_4[int(rng.integers(0, len(SIZES_4)))])
    stamps = int(rng.integers(5, 21))
    density = float(rng.uniform(0.002, 0.01))
    ratio = float(rng.uniform(1.1, 1.8))
    return dict(size=size, stamps=stamps, density=density, ratio=ratio,
                n_src=int(round(density * size * size)))


def make_pair4(frame, dtype=np.float32):
    """Pair `frame` of preset 4: (template, science, info); info carries the
    pair's stamp grid and threshHigh."""
    d = config4_draw(frame)
    lo, hi = CONFIGS[2]["fwhm_t"]
    T, S, info = make_pair(2, frame=frame, size=d["size"], n_src=d["n_src"], dtype=dtype,
                           seed=4, stamps=d["stamps"], chunk=16384,
                           fwhm_s=(lo * d["ratio"], hi * d["ratio"]))
    info.update(config=4, density=d["density"], fwhm_ratio=d["ratio"])
    return T, S, info
