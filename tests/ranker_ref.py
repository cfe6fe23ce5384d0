"""NumPy FP64 restatement of the substamp ranker network of xb_ranker.cu
(test infrastructure: the checker of the CUDA forward and backward kernels).

Parameter layout: conv1 w [8,2,5,5] b [8] | conv2 w [8,8,3,3] b [8] |
conv3 w [8,8,3,3] b [8] | mlp w [32,16] b [32] | head w [40] b [1].
"""
import numpy as np
from numpy.lib.stride_tricks import sliding_window_view as swv

SHAPES = [("c1w", (8, 2, 5, 5)), ("c1b", (8,)), ("c2w", (8, 8, 3, 3)), ("c2b", (8,)),
          ("c3w", (8, 8, 3, 3)), ("c3b", (8,)), ("m1w", (32, 16)), ("m1b", (32,)),
          ("hw", (40,)), ("hb", (1,))]


def bf16(w):
    """The weights as the network uses them: each FP32 value rounded to BF16
    (nearest, ties to even), returned as float64."""
    u = np.ascontiguousarray(w, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(w):
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = np.asarray(w[o:o + n], np.float64).reshape(shp)
        o += n
    assert o == len(w)
    return out


def pack(d):
    return np.concatenate([d[name].reshape(-1) for name, _ in SHAPES])


def _conv(x, w, b, stride):
    k = w.shape[-1]
    win = swv(x, (k, k), axis=(1, 2))[:, ::stride, ::stride]   # (ci, y, x, k, k)
    return np.einsum("oikl,iyxkl->oyx", w, win) + b[:, None, None]


def forward(w, st, px):
    """Logit and activations of one sample (st: 16, px: 2x31x31)."""
    P = unpack(w)
    x = np.asarray(px, np.float64)
    z1 = _conv(x, P["c1w"], P["c1b"], 2)
    a1 = np.maximum(z1, 0)
    z2 = _conv(a1, P["c2w"], P["c2b"], 2)
    a2 = np.maximum(z2, 0)
    z3 = _conv(a2, P["c3w"], P["c3b"], 1)
    a3 = np.maximum(z3, 0)
    pool = a3.mean(axis=(1, 2))
    zm = P["m1w"] @ np.asarray(st, np.float64) + P["m1b"]
    hm = np.maximum(zm, 0)
    hid = np.concatenate([pool, hm])
    logit = float(P["hw"] @ hid + P["hb"][0])
    return logit, dict(x=x, a1=a1, a2=a2, a3=a3, hid=hid, st=np.asarray(st, np.float64), P=P)


def _conv_back(dz, xin, w, stride):
    """Gradients of a strided valid convolution: dW, db, dx."""
    k = w.shape[-1]
    win = swv(xin, (k, k), axis=(1, 2))[:, ::stride, ::stride]
    dw = np.einsum("oyx,iyxkl->oikl", dz, win)
    db = dz.sum(axis=(1, 2))
    dx = np.zeros_like(xin)
    Y, X = dz.shape[1:]
    for ky in range(k):
        for kx in range(k):
            dx[:, ky:ky + stride * Y:stride, kx:kx + stride * X:stride] += np.einsum(
                "oyx,oi->iyx", dz, w[:, :, ky, kx])
    return dw, db, dx


def grad(w, st, px, y, sw=1.0):
    """Loss sw * BCE(sigmoid(z), y) and its gradient (packed like w)."""
    z, A = forward(w, st, px)
    P = A["P"]
    p = 1.0 / (1.0 + np.exp(-z))
    loss = sw * (max(z, 0.0) - z * y + np.log1p(np.exp(-abs(z))))
    dz = sw * (p - y)
    G = {"hw": dz * A["hid"], "hb": np.array([dz])}
    dh = dz * P["hw"]
    dzm = dh[8:] * (A["hid"][8:] > 0)
    G["m1w"] = np.outer(dzm, A["st"])
    G["m1b"] = dzm
    d3 = (dh[:8] / 16.0)[:, None, None] * (A["a3"] > 0)
    G["c3w"], G["c3b"], da2 = _conv_back(d3, A["a2"], P["c3w"], 1)
    d2 = da2 * (A["a2"] > 0)
    G["c2w"], G["c2b"], da1 = _conv_back(d2, A["a1"], P["c2w"], 2)
    d1 = da1 * (A["a1"] > 0)
    G["c1w"], G["c1b"], _ = _conv_back(d1, A["x"], P["c1w"], 2)
    return loss, pack(G)
