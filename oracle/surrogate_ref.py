"""CPU reference of the plasma surrogate network (test infrastructure only:
the checker of the CUDA forward and backward kernels, never a product
path).  Same architecture and numerics as the device: weights and
hidden activations rounded to BF16 (round to nearest even), the output
layer left unrounded, products accumulated in FP64 here (FP32 on the
device), tanh after layers 0-2, "same" padding.

Layer l maps ci_l -> co_l channels: 3 -> 64 -> 64 -> 64 -> 1, kernel 9.
Parameters (FP32, the layout of fil_nn_get_params): per layer the weights
[co][ci][k] followed by the bias [co]."""
import numpy as np

CH, K, HALF = 64, 9, 4
CI = [3, CH, CH, CH]
CO = [CH, CH, CH, 1]


def nparams():
    return sum(co * ci * K + co for ci, co in zip(CI, CO))


def bf16(x):
    """Round FP32 values to BF16 (nearest, ties to even), returned as FP64."""
    u = np.asarray(x, dtype=np.float32).view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    out, o = [], 0
    for ci, co in zip(CI, CO):
        w = np.asarray(p[o:o + co * ci * K], dtype=np.float64).reshape(co, ci, K)
        o += co * ci * K
        b = np.asarray(p[o:o + co], dtype=np.float64)
        o += co
        out.append((w, b))
    return out


def conv(x, w):
    """y[b][co][t] = sum_ci,k w[co][ci][k] x[b][ci][t + k - 4], zero outside."""
    B, C, T = x.shape
    xp = np.zeros((B, C, T + 2 * HALF))
    xp[:, :, HALF:HALF + T] = x
    y = np.zeros((B, w.shape[0], T))
    for k in range(K):
        y += np.einsum("oc,bct->bot", w[:, :, k], xp[:, :, k:k + T])
    return y


def conv_t(g, w):
    """Input gradient of conv: dx[b][ci][t] = sum_co,k w[co][ci][k] g[b][co][t - k + 4]."""
    B, C, T = g.shape
    gp = np.zeros((B, C, T + 2 * HALF))
    gp[:, :, HALF:HALF + T] = g
    dx = np.zeros((B, w.shape[1], T))
    for k in range(K):
        dx += np.einsum("oc,bot->bct", w[:, :, k], gp[:, :, 2 * HALF - k:2 * HALF - k + T])
    return dx


def forward(p, feat):
    """Activations [x0, y0, y1, y2, out] as the device stores them (BF16
    inputs and hidden layers, unrounded output)."""
    layers = unpack(p)
    acts = [bf16(feat)]
    for l, (w, b) in enumerate(layers):
        y = conv(acts[-1], bf16(w)) + b[None, :, None]
        acts.append(bf16(np.tanh(y)) if l < 3 else y)
    return acts


def grad(p, feat, tgt, mask):
    """(loss, gradient of the FP32 parameters) of the weighted squared
    error sum m (out - tgt)^2 / sum m."""
    layers = unpack(p)
    acts = forward(p, feat)
    out = acts[-1][:, 0, :]
    cnt = mask.sum()
    e = out - tgt
    loss = float((mask * e * e).sum() / cnt)
    g = (2.0 * mask * e / cnt)[:, None, :]
    grads = [None] * 4
    for l in range(3, -1, -1):
        w, _ = layers[l]
        x = acts[l]
        B, C, T = x.shape
        xp = np.zeros((B, C, T + 2 * HALF))
        xp[:, :, HALF:HALF + T] = x
        dw = np.stack([np.einsum("bot,bct->oc", g, xp[:, :, k:k + T]) for k in range(K)], axis=2)
        db = g.sum(axis=(0, 2))
        grads[l] = (dw, db)
        if l > 0:
            dx = conv_t(g, bf16(w))
            g = dx * (1.0 - acts[l] ** 2)
    flat = []
    for dw, db in grads:
        flat.append(dw.reshape(-1))
        flat.append(db)
    return loss, np.concatenate(flat)
