"""Learned substamp ranker: training data from the plain ksc loop, training on
the GPU through the library's kernels (xb_ranker_grad / xb_ranker_adam), and
use in a pipeline (xb_ranker_set + option "rank").

Labels.  After sss, every stamp holds up to maxSS candidate substamps in the
reference's order (brightest first); ksc uses them in that order and moves to
the next one each time the fit rejects the current one.  For the stamp set
the fit runs on, a candidate before the final one is a rejection (label 0),
the final one, if any remains, was accepted (label 1), later ones were never
tried (no label).  Features are taken right after sss, where the pipeline
scores them.
"""
import ctypes

import numpy as np

from . import XB_MODE_PLAIN, Context, XbError, lib

NSTAT = 16
WIN = 31
NPIX = 2 * WIN * WIN


def param_count():
    return int(lib().xb_ranker_param_count())


def init_weights(seed=0):
    """He-normal weights for the ReLU layers, small head, zero biases (the
    layout of xb_ranker.cu)."""
    rng = np.random.default_rng(seed)
    parts = [
        rng.normal(0, np.sqrt(2 / 50), 8 * 2 * 25), np.zeros(8),     # conv1
        rng.normal(0, np.sqrt(2 / 72), 8 * 8 * 9), np.zeros(8),      # conv2
        rng.normal(0, np.sqrt(2 / 72), 8 * 8 * 9), np.zeros(8),      # conv3
        rng.normal(0, np.sqrt(2 / 16), 32 * 16), np.zeros(32),       # mlp
        rng.normal(0, 0.1, 40), np.zeros(1),                         # head
    ]
    w = np.concatenate(parts).astype(np.float32)
    assert w.size == param_count()
    return w


def features(ctx, stamp_set):
    """(stats n x 16, pix n x 2 x 31 x 31, stamp n, slot n) of every candidate
    substamp of a stamp set, after ctx.sss()."""
    L = lib()
    n = ctypes.c_int(0)
    rc = L.xb_ranker_features(ctx.h, stamp_set, None, None, None, None, 0, ctypes.byref(n))
    if rc:
        raise XbError(rc, L.xb_last_error(ctx.h).decode())
    m = n.value
    st = np.empty((m, NSTAT), np.float32)
    px = np.empty((m, 2, WIN, WIN), np.float32)
    stamp = np.empty(m, np.int32)
    slot = np.empty(m, np.int32)
    rc = L.xb_ranker_features(ctx.h, stamp_set, st.ctypes.data, px.ctypes.data, stamp.ctypes.data,
                              slot.ctypes.data, m, ctypes.byref(n))
    if rc:
        raise XbError(rc, L.xb_last_error(ctx.h).decode())
    return st, px, stamp, slot


def labelled_frame(T, S, params):
    """Runs the plain pipeline up to ksc on one pair; returns the labelled
    candidates (stats, pix, labels) of the fitted stamp set and the number of
    ksc iterations."""
    p = type(params).from_buffer_copy(params)
    p.mode = XB_MODE_PLAIN
    ctx = Context(p, trace=True)
    ctx.init(T, S)
    ctx.sss()
    feats = [features(ctx, si) for si in (0, 1)]
    ctx.cmv()
    ctx.cd()
    ctx.ksc()
    si = 0 if int(ctx.scalar("convTemplate")) else 1
    cur = ctx.array("cur", np.int32)
    count = ctx.array("ss_count%d" % si, np.int32)
    st, px, stamp, slot = feats[si]
    lab = np.full(len(stamp), -1, np.int8)
    for i, (s, k) in enumerate(zip(stamp, slot)):
        if k < cur[s]:
            lab[i] = 0
        elif k == cur[s] and cur[s] < count[s]:
            lab[i] = 1
    keep = lab >= 0
    return st[keep], px[keep], lab[keep].astype(np.float32), int(ctx.scalar("ksc_iterations"))


def train(stats, pix, labels, epochs=40, batch=256, lr=3e-3, seed=0, weights=None,
          balance=True, log=None):
    """Adam on the weighted binary cross-entropy, on the GPU.  Returns the
    trained weights (numpy FP32) and the per-epoch mean loss."""
    import torch
    L = lib()
    P = param_count()
    n = len(labels)
    dev = torch.device("cuda")
    X_st = torch.from_numpy(np.ascontiguousarray(stats, np.float32)).to(dev)
    X_px = torch.from_numpy(np.ascontiguousarray(pix, np.float32).reshape(n, NPIX)).to(dev)
    y = torch.from_numpy(np.ascontiguousarray(labels, np.float32)).to(dev)
    sw = torch.ones(n, dtype=torch.float32, device=dev)
    if balance:
        pos = float(labels.mean())
        if 0 < pos < 1:
            sw = torch.where(y > 0.5, 0.5 / pos, 0.5 / (1 - pos)).float()
    W = torch.from_numpy(weights if weights is not None else init_weights(seed)).to(dev)
    m = torch.zeros(P, device=dev)
    v = torch.zeros(P, device=dev)
    g = torch.zeros(P, device=dev)
    gper = torch.empty((batch, P), device=dev)
    loss = torch.empty(batch, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    gen = torch.Generator(device="cpu").manual_seed(seed)
    step = 0
    history = []
    for ep in range(epochs):
        perm = torch.randperm(n, generator=gen).to(dev)
        tot = 0.0
        for b0 in range(0, n, batch):
            idx = perm[b0:b0 + batch]
            nb = len(idx)
            bs, bp, by, bw = (X_st[idx].contiguous(), X_px[idx].contiguous(), y[idx].contiguous(),
                              sw[idx].contiguous())
            rc = L.xb_ranker_grad(W.data_ptr(), bs.data_ptr(), bp.data_ptr(), by.data_ptr(),
                                  bw.data_ptr(), nb, gper.data_ptr(), g.data_ptr(), loss.data_ptr(),
                                  stream)
            if rc:
                raise XbError(rc, "xb_ranker_grad")
            step += 1
            rc = L.xb_ranker_adam(W.data_ptr(), g.data_ptr(), m.data_ptr(), v.data_ptr(), step,
                                  ctypes.c_float(lr), stream)
            if rc:
                raise XbError(rc, "xb_ranker_adam")
            tot += float(loss[:nb].sum())
        history.append(tot / n)
        if log:
            log(ep, history[-1])
    return W.cpu().numpy(), history


def logits(weights, stats, pix):
    """Scores of candidates with the library's inference kernel."""
    import torch
    L = lib()
    n = len(stats)
    dev = torch.device("cuda")
    W = torch.from_numpy(np.ascontiguousarray(weights, np.float32)).to(dev)
    bs = torch.from_numpy(np.ascontiguousarray(stats, np.float32)).to(dev)
    bp = torch.from_numpy(np.ascontiguousarray(pix, np.float32).reshape(n, NPIX)).to(dev)
    out = torch.empty(n, device=dev)
    rc = L.xb_ranker_forward(W.data_ptr(), bs.data_ptr(), bp.data_ptr(), n, out.data_ptr(),
                             torch.cuda.current_stream().cuda_stream)
    if rc:
        raise XbError(rc, "xb_ranker_forward")
    return out.cpu().numpy()


def enable(ctx, weights, policy=1, tau=0.5):
    """Loads the weights into a context and turns ranking on (policy 1:
    demote candidates below accept probability tau; 2: sort by score)."""
    w = np.ascontiguousarray(weights, np.float32)
    L = lib()
    rc = L.xb_ranker_set(ctx.h, w.ctypes.data, w.size)
    if rc:
        raise XbError(rc, L.xb_last_error(ctx.h).decode())
    ctx.set_option("rank", policy)
    ctx.set_option("rank_tau", int(round(tau * 1000)))


def preset5_weights():
    """The shipped weights (xbach/ranker_preset5.npy, made by
    `python -m xbach.train_ranker`): trained on preset-5 defect fields."""
    import pathlib
    return np.load(pathlib.Path(__file__).resolve().parent / "ranker_preset5.npy")
