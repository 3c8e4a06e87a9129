"""FP64 forward and backward of the distilled student net (numpy).

TEST INFRASTRUCTURE ONLY: the checker for the GPU training kernels
(lg_student_grads / lg_student_train_step); the product never imports it.

The student: 5x5 conv c_in -> W, n3x3 x 3x3 conv W -> W, ReLU after each;
policy head 1x1 W -> 1 (no activation) -> softmax over 361; value head 1x1
W -> 1 -> FC 361 -> H (ReLU) -> FC H -> 1 -> tanh.  Convs use the reference's
'same'-padded im2col formulation (Im2Col.h:9-50, Network.cpp:345-393).
Loss = mean over the batch of KL(t || softmax(logits)) + vw * (v - vt)^2.

Flat parameter layout: per conv W[O][C][k][k], b[O]; wp[W], bp; wv[W], bv;
W1[H][361], b1[H], W2[H], b2.
"""
from __future__ import annotations

import numpy as np

P = 361


def shapes(c_in, width, n3x3, H):
    out = []
    for l in range(n3x3 + 1):
        k = 5 if l == 0 else 3
        cin = c_in if l == 0 else width
        out.append(("conv", k, cin, width))
    out += [("wp", width), ("bp", 1), ("wv", width), ("bv", 1), ("W1", H * P), ("b1", H),
            ("W2", H), ("b2", 1)]
    return out


def param_count(c_in, width, n3x3, H):
    n = 0
    for s in shapes(c_in, width, n3x3, H):
        n += s[3] * s[2] * s[1] * s[1] + s[3] if s[0] == "conv" else s[1]
    return n


def unpack(params, c_in, width, n3x3, H):
    p = np.asarray(params, dtype=np.float64)
    off = 0
    convs, heads = [], {}
    for s in shapes(c_in, width, n3x3, H):
        if s[0] == "conv":
            _, k, cin, cout = s
            n = cout * cin * k * k
            W = p[off:off + n].reshape(cout, cin, k, k)
            off += n
            b = p[off:off + cout]
            off += cout
            convs.append((W, b))
        else:
            heads[s[0]] = p[off:off + s[1]]
            off += s[1]
    heads["W1"] = heads["W1"].reshape(H, P)
    return convs, heads


def im2col(x, k):
    """x [B][C][19][19] -> [B][C*k*k][361], 'same' zero padding, row order
    (c, ky, kx) as Im2Col.h."""
    B, C = x.shape[:2]
    pad = k // 2
    xp = np.zeros((B, C, 19 + 2 * pad, 19 + 2 * pad), dtype=x.dtype)
    xp[:, :, pad:pad + 19, pad:pad + 19] = x
    cols = np.empty((B, C, k, k, 19, 19), dtype=x.dtype)
    for ky in range(k):
        for kx in range(k):
            cols[:, :, ky, kx] = xp[:, :, ky:ky + 19, kx:kx + 19]
    return cols.reshape(B, C * k * k, P)


def col2im(cols, C, k):
    """Adjoint of im2col: [B][C*k*k][361] -> [B][C][19][19]."""
    B = cols.shape[0]
    pad = k // 2
    c6 = cols.reshape(B, C, k, k, 19, 19)
    xp = np.zeros((B, C, 19 + 2 * pad, 19 + 2 * pad), dtype=cols.dtype)
    for ky in range(k):
        for kx in range(k):
            xp[:, :, ky:ky + 19, kx:kx + 19] += c6[:, :, ky, kx]
    return xp[:, :, pad:pad + 19, pad:pad + 19]


def forward(params, planes, c_in, width, n3x3, H):
    convs, hd = unpack(params, c_in, width, n3x3, H)
    x = np.asarray(planes, dtype=np.float64).reshape(-1, c_in, 19, 19)
    cache = []
    for W, b in convs:
        k = W.shape[2]
        col = im2col(x, k)
        y = np.einsum("ok,bkp->bop", W.reshape(W.shape[0], -1), col) + b[None, :, None]
        y = np.maximum(y, 0.0)
        cache.append((x, col, y))
        x = y.reshape(-1, W.shape[0], 19, 19)
    X = x.reshape(x.shape[0], width, P)
    logits = np.einsum("bcp,c->bp", X, hd["wp"]) + hd["bp"][0]
    x361 = np.einsum("bcp,c->bp", X, hd["wv"]) + hd["bv"][0]
    hid = np.maximum(x361 @ hd["W1"].T + hd["b1"][None, :], 0.0)
    v = np.tanh(hid @ hd["W2"] + hd["b2"][0])
    return dict(convs=convs, hd=hd, cache=cache, X=X, logits=logits, x361=x361, hid=hid, v=v)


def softmax(x):
    e = np.exp(x - x.max(axis=1, keepdims=True))
    return e / e.sum(axis=1, keepdims=True)


def loss_and_grads(params, planes, target, vt, vw, c_in, width, n3x3, H):
    f = forward(params, planes, c_in, width, n3x3, H)
    B = f["logits"].shape[0]
    t = np.asarray(target, dtype=np.float64)
    vt = np.asarray(vt, dtype=np.float64)
    s = softmax(f["logits"])
    logq = np.log(s)
    kl = np.where(t > 0, t * (np.log(np.where(t > 0, t, 1.0)) - logq), 0.0).sum() / B
    d = f["v"] - vt
    lv = (d * d).sum() / B
    hd = f["hd"]
    dlogits = (s - t) / B
    du = 2.0 * vw * d * (1.0 - f["v"] ** 2) / B
    dhid = du[:, None] * hd["W2"][None, :]
    dpre = dhid * (f["hid"] > 0)
    g = {}
    g["W2"] = (du[:, None] * f["hid"]).sum(0)
    g["b2"] = np.array([du.sum()])
    g["W1"] = dpre.T @ f["x361"]
    g["b1"] = dpre.sum(0)
    dx361 = dpre @ hd["W1"]
    X = f["X"]
    g["wp"] = np.einsum("bp,bcp->c", dlogits, X)
    g["bp"] = np.array([dlogits.sum()])
    g["wv"] = np.einsum("bp,bcp->c", dx361, X)
    g["bv"] = np.array([dx361.sum()])
    dX = dlogits[:, None, :] * hd["wp"][None, :, None] + dx361[:, None, :] * hd["wv"][None, :, None]
    conv_grads = []
    dY = dX
    for (W, b), (x, col, y) in zip(reversed(f["convs"]), reversed(f["cache"])):
        O, C, k, _ = W.shape
        dYp = dY.reshape(-1, O, P) * (y > 0)
        dW = np.einsum("bop,bkp->ok", dYp, col).reshape(W.shape)
        db = dYp.sum(axis=(0, 2))
        dcol = np.einsum("ok,bop->bkp", W.reshape(O, -1), dYp)
        dY = col2im(dcol, C, k).reshape(-1, C, P)
        conv_grads.append((dW, db))
    conv_grads.reverse()
    flat = []
    for dW, db in conv_grads:
        flat += [dW.ravel(), db]
    for name in ("wp", "bp", "wv", "bv", "W1", "b1", "W2", "b2"):
        flat.append(np.asarray(g[name]).ravel())
    return (kl, lv), np.concatenate(flat)
