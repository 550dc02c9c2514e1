"""The CPU restatement of the warm-start network checks itself: its
analytic gradients against central finite differences (FP64, no BF16
rounding), so that it can serve as the reference for the CUDA gradients."""
import numpy as np

from oracle import unet_oracle as U


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    n, B = 8, 1
    w, b, hoff, total = U.layout()
    p = np.zeros(total)
    for l, (cin, cout, _) in enumerate(U.CONVS):
        real = 4 if l == 0 else cin
        W = rng.normal(0, np.sqrt(2 / (27 * real)), (27, cin, cout))
        W[:, real:, :] = 0
        p[w[l]:w[l] + W.size] = W.ravel()
        p[b[l]:b[l] + cout] = rng.normal(0, 0.05, cout)
    p[hoff:hoff + 16] = rng.normal(0, 0.3, 16)
    A = (rng.random((B, n, n, n)) < 0.6).astype(np.uint8)
    bb = rng.normal(0, 1, (B, n, n, n)).astype(np.float32)
    x0 = rng.normal(0, 1e-3, (B, n, n, n)).astype(np.float32)
    x = rng.normal(0, 1e-3, (B, n, n, n)).astype(np.float32)
    r0 = rng.normal(0, 1, (B, n, n, n)).astype(np.float32)
    _, g, _ = U.loss_and_grads(p, A, bb, x0, r0, x)
    idx = list(rng.choice(total, 12, replace=False)) + [hoff + 3, hoff + 16, b[0] + 1,
                                                        w[13] + 100, w[8] + 5000]
    for i in idx:
        e = 1e-5
        pp, pm = p.copy(), p.copy()
        pp[i] += e
        pm[i] -= e
        fd = (U.loss_and_grads(pp, A, bb, x0, r0, x)[0] -
              U.loss_and_grads(pm, A, bb, x0, r0, x)[0]) / (2 * e)
        assert abs(fd - g[i]) <= 1e-5 * (abs(fd) + abs(g[i])) + 1e-12, (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    x = np.array([1.0, 1.00390625, 1.01171875, -2.5, 3.0e-5], np.float32)
    r = U.bf16(x)
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.015625 and r[3] == -2.5
    assert abs(r[4] - 3.0e-5) <= 3.0e-5 * 2 ** -8


def test_prolongation_and_pooled_targets():
    """Trilinear prolongation keeps constants and reproduces linear fields
    away from the clamped boundary; pooled targets average liquid cells
    only."""
    from oracle import unet_oracle as U
    c = np.full((1, 4, 4, 4), 2.5)
    assert np.allclose(U.prolong(c, 2), 2.5)
    i = np.arange(4, dtype=float)
    lin = (i[:, None, None] + 0 * i[None, :, None] + 0 * i[None, None, :])[None]
    up = U.prolong(lin, 1)[0]
    fine = (np.arange(8) + 0.5) / 2 - 0.5
    assert np.allclose(up[1:-1, 3, 3], fine[1:-1])
    A = np.zeros((1, 4, 4, 4), np.uint8)
    A[0, 0, 0, 0] = 1
    A[0, 1, 1, 1] = 1
    x = np.zeros((1, 4, 4, 4), np.float32)
    x[0, 0, 0, 0], x[0, 1, 1, 1], x[0, 0, 1, 0] = 2.0, 4.0, 100.0
    Ac, xc, _ = U.pool_target(A, x, x, 1)
    assert Ac[0, 0, 0, 0] == 1 and Ac.sum() == 1
    assert xc[0, 0, 0, 0] == 3.0
