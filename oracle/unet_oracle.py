"""CPU restatement of the learned warm start's network (numpy, FP64).

TEST INFRASTRUCTURE ONLY: the checker for the CUDA U-Net in
flip3d_gb300/csrc/k_unet.cu (forward, backward, loss). It follows the same
layer order, parameter layout and feature/target scaling; with
`bf16=True` it rounds weights and every stored activation and gradient to
BF16 at the points where the CUDA code stores BF16, so the remaining
differences come from FP32 accumulation order alone.

Arrays are [batch, i, j, k, channel] with cells x-major like the solver's
grids; taps are numbered (dz*3 + dy)*3 + dx with dz along i and dx along k.
"""
from __future__ import annotations

import numpy as np

CONVS = [(16, 16, 0), (16, 16, 0), (16, 32, 1), (32, 32, 1), (32, 48, 2), (48, 48, 2),
         (48, 64, 3), (64, 64, 3), (112, 48, 2), (48, 48, 2), (80, 32, 1), (32, 32, 1),
         (48, 16, 0), (16, 16, 0)]


def layout():
    """Offsets of each conv's W [27][cin][cout] and b [cout], then the head."""
    off, w, b = 0, [], []
    for cin, cout, _ in CONVS:
        w.append(off)
        off += 27 * cin * cout
        b.append(off)
        off += cout
    return w, b, off, off + 17


def unpack(p):
    w, b, hoff, total = layout()
    assert p.shape[0] == total
    W = [p[w[l]:w[l] + 27 * c[0] * c[1]].reshape(27, c[0], c[1]) for l, c in enumerate(CONVS)]
    B = [p[b[l]:b[l] + c[1]] for l, c in enumerate(CONVS)]
    return W, B, p[hoff:hoff + 16], p[hoff + 16]


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def conv(X, W, b=None):
    """3x3x3 'same' convolution with zero padding; X [B,n,n,n,Cin]."""
    Bn, n = X.shape[0], X.shape[1]
    Xp = np.zeros((Bn, n + 2, n + 2, n + 2, X.shape[4]))
    Xp[:, 1:-1, 1:-1, 1:-1] = X
    Y = np.zeros((Bn, n, n, n, W.shape[2]))
    for t in range(27):
        dz, dy, dx = t // 9, (t // 3) % 3, t % 3
        Y += Xp[:, dz:dz + n, dy:dy + n, dx:dx + n] @ W[t]
    if b is not None:
        Y += b
    return Y


def conv_wgrad(X, dZ):
    Bn, n = X.shape[0], X.shape[1]
    Xp = np.zeros((Bn, n + 2, n + 2, n + 2, X.shape[4]))
    Xp[:, 1:-1, 1:-1, 1:-1] = X
    gW = np.zeros((27, X.shape[4], dZ.shape[4]))
    for t in range(27):
        dz, dy, dx = t // 9, (t // 3) % 3, t % 3
        xs = Xp[:, dz:dz + n, dy:dy + n, dx:dx + n].reshape(-1, X.shape[4])
        gW[t] = xs.T @ dZ.reshape(-1, dZ.shape[4])
    return gW, dZ.reshape(-1, dZ.shape[4]).sum(axis=0)


def conv_dgrad(dZ, W):
    """Transposed convolution: the 'same' convolution with flipped taps and
    transposed channel matrices."""
    Wt = np.stack([W[26 - t].T for t in range(27)])
    return conv(dZ, Wt)


def pool(X):
    Bn, n, C = X.shape[0], X.shape[1], X.shape[4]
    return X.reshape(Bn, n // 2, 2, n // 2, 2, n // 2, 2, C).mean(axis=(2, 4, 6))


def up(X):
    return X.repeat(2, axis=1).repeat(2, axis=2).repeat(2, axis=3)


def up_bwd(dU):
    Bn, n, C = dU.shape[0], dU.shape[1], dU.shape[4]
    return dU.reshape(Bn, n // 2, 2, n // 2, 2, n // 2, 2, C).sum(axis=(2, 4, 6))


def pool_bwd(dP):
    return up(dP) / 8.0


def features(A, b, x0, r0):
    """A, b, x0, r0: [B, n, n, n]; returns the 16-channel input (mask,
    r0/s_r, b/s_b, x0/s_x), the target scale s_t = s_r h^2 per sample and
    the liquid mask (flip3d_gb300/csrc/k_unet.cu k_sample_scale, k_features)."""
    Bn, n = A.shape[0], A.shape[1]
    fl = A == 1
    X = np.zeros(A.shape + (16,))
    st = np.ones(Bn)
    for s in range(Bn):
        c = fl[s].sum()

        def rms(a):
            ss = float((a[s][fl[s]].astype(np.float64) ** 2).sum())
            return np.sqrt(ss / c) if c > 0 and ss > 0 else 1.0
        sb, sr, sx = rms(b), rms(r0), rms(x0)
        st[s] = np.float32(sr / (n * n))
        X[s, ..., 0] = fl[s]
        X[s, ..., 1] = np.where(fl[s], np.float32(r0[s]) / np.float32(sr), 0)
        X[s, ..., 2] = np.where(fl[s], np.float32(b[s]) / np.float32(sb), 0)
        X[s, ..., 3] = np.where(fl[s], np.float32(x0[s]) / np.float32(sx), 0)
    return X, st, fl


def pool_features(X, levels, round_bf16=False):
    """The 16-channel input average-pooled `levels` times (rounded to BF16
    after every pooling, as k_pool stores it)."""
    r = bf16 if round_bf16 else (lambda a: a)
    X = r(X)
    for _ in range(levels):
        X = r(pool(X))
    return X


def pool_target(A, x, x0, levels):
    """Coarse liquid flags and the liquid-cell averages of x and x0 over
    each (2^levels)^3 block (flip3d_gb300/csrc/k_unet.cu k_pool_target)."""
    f = 1 << levels
    Bn, n = A.shape[0], A.shape[1]
    m = n // f
    fl = (A == 1).reshape(Bn, m, f, m, f, m, f)
    cnt = fl.sum(axis=(2, 4, 6))

    def avg(a):
        a32 = np.float32(a).astype(np.float64).reshape(Bn, m, f, m, f, m, f)
        s = np.where(fl, a32, 0.0).sum(axis=(2, 4, 6))
        return np.where(cnt > 0, s / np.maximum(cnt, 1), 0.0)
    Ac = np.where(cnt > 0, 1, 0).astype(np.uint8)
    return Ac, avg(x), avg(x0)


def prolong(O, levels):
    """Trilinear prolongation of a cell-centred [B, m, m, m] field to
    (m 2^levels)^3, clamped at the boundary (k_prolong)."""
    f = 1 << levels
    m = O.shape[1]
    n = m * f
    xc = (np.arange(n) + 0.5) / f - 0.5
    lo = np.floor(xc).astype(int)
    w = xc - lo
    a = np.clip(lo, 0, m - 1)
    b = np.clip(lo + 1, 0, m - 1)
    out = O
    for axis in (1, 2, 3):
        shp = [1, 1, 1, 1]
        shp[axis] = n
        wa = (1.0 - w).reshape(shp)
        wb = w.reshape(shp)
        out = np.take(out, a, axis=axis) * wa + np.take(out, b, axis=axis) * wb
    return out


def forward(p, X, round_bf16=False):
    W, Bs, wh, bh = unpack(np.asarray(p, np.float64))
    r = bf16 if round_bf16 else (lambda a: a)
    if round_bf16:
        W = [bf16(w) for w in W]
    t = {"X0": r(X)}

    def cv(l, x):
        return r(np.maximum(conv(x, W[l], Bs[l]), 0.0))
    t["A0"] = cv(0, t["X0"]); t["E0"] = cv(1, t["A0"])
    t["P1"] = r(pool(t["E0"])); t["A1"] = cv(2, t["P1"]); t["E1"] = cv(3, t["A1"])
    t["P2"] = r(pool(t["E1"])); t["A2"] = cv(4, t["P2"]); t["E2"] = cv(5, t["A2"])
    t["P3"] = r(pool(t["E2"])); t["A3"] = cv(6, t["P3"]); t["E3"] = cv(7, t["A3"])
    t["U2"] = np.concatenate([up(t["E3"]), t["E2"]], axis=4)
    t["B2"] = cv(8, t["U2"]); t["D2"] = cv(9, t["B2"])
    t["U1"] = np.concatenate([up(t["D2"]), t["E1"]], axis=4)
    t["B1"] = cv(10, t["U1"]); t["D1"] = cv(11, t["B1"])
    t["U0"] = np.concatenate([up(t["D1"]), t["E0"]], axis=4)
    t["B0"] = cv(12, t["U0"]); t["D0"] = cv(13, t["B0"])
    t["O"] = t["D0"] @ wh + bh
    return t


def loss_and_grads(p, A, b, x0, r0, x, round_bf16=False, levels=0):
    """Loss (mean squared error over liquid cells of the batch) and its
    gradient with respect to the flat parameter vector. With `levels` > 0
    the network sees the pooled features and the loss compares it with the
    pooled targets on the coarse grid."""
    X, sx, fl = features(A, b, x0, r0)
    if levels:
        X = pool_features(X, levels, round_bf16)
        A, x, x0 = pool_target(A, x, x0, levels)
        fl = A == 1
    t = forward(p, X, round_bf16)
    W, Bs, wh, bh = unpack(np.asarray(p, np.float64))
    r = bf16 if round_bf16 else (lambda a: a)
    if round_bf16:
        W = [bf16(w) for w in W]
    T = (np.float32(x) - np.float32(x0)) / sx[:, None, None, None]
    cnt = fl.sum()
    e = np.where(fl, t["O"] - T, 0.0)
    loss = float((e ** 2).sum() / cnt)
    dO = 2.0 * e / cnt
    g = np.zeros_like(np.asarray(p, np.float64))
    woff, boff, hoff, _ = layout()
    g[hoff:hoff + 16] = (t["D0"] * dO[..., None]).reshape(-1, 16).sum(axis=0)
    g[hoff + 16] = dO.sum()
    dY = r(dO[..., None] * wh)

    def back(l, dY, Xin, Yout, want_dx=True):
        dZ = r(np.where(Yout > 0, dY, 0.0))
        gW, gb = conv_wgrad(Xin, dZ)
        cin, cout, _ = CONVS[l]
        g[woff[l]:woff[l] + 27 * cin * cout] = gW.ravel()
        g[boff[l]:boff[l] + cout] = gb
        return r(conv_dgrad(dZ, W[l])) if want_dx else None

    d = back(13, dY, t["B0"], t["D0"])
    dU0 = back(12, d, t["U0"], t["B0"])
    S0 = dU0[..., 32:48]
    d = r(up_bwd(dU0[..., :32]))
    d = back(11, d, t["B1"], t["D1"])
    dU1 = back(10, d, t["U1"], t["B1"])
    S1 = dU1[..., 48:80]
    d = r(up_bwd(dU1[..., :48]))
    d = back(9, d, t["B2"], t["D2"])
    dU2 = back(8, d, t["U2"], t["B2"])
    S2 = dU2[..., 64:112]
    d = r(up_bwd(dU2[..., :64]))
    d = back(7, d, t["A3"], t["E3"])
    d = back(6, d, t["P3"], t["A3"])
    d = r(pool_bwd(d) + S2)
    d = back(5, d, t["A2"], t["E2"])
    d = back(4, d, t["P2"], t["A2"])
    d = r(pool_bwd(d) + S1)
    d = back(3, d, t["A1"], t["E1"])
    d = back(2, d, t["P1"], t["A1"])
    d = r(pool_bwd(d) + S0)
    d = back(1, d, t["A0"], t["E0"])
    back(0, d, t["X0"], t["A0"], want_dx=False)
    return loss, g, t
