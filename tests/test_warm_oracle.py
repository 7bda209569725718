"""The warm-start oracle on the CPU: its analytic gradient against central
finite differences (FP64, no BF16 emulation), its push against a dense
power-series restatement, and its least-squares fit against numpy's."""
import numpy as np

from graphops_gb300 import gen
from oracle import warm_oracle as wo


def small_case(n=60, seed=0):
    g = gen.erdos_renyi(n, 0.08, 0.05, seed=seed)
    rng = np.random.default_rng(seed)
    in_rp, in_col = wo.in_csr(n, g.row_ptr, g.col)
    x1 = np.zeros((n, wo.W_IN))
    x1[:, :36] = rng.standard_normal((n, 36))
    x1[:, 36] = 1.0
    params = np.zeros(wo.P_COUNT)
    params[wo.P_W1:wo.P_W2] = 0.2 * rng.standard_normal(wo.W_IN * wo.HIDDEN)
    params[wo.P_W1 + 37 * wo.HIDDEN:wo.P_W2] = 0.0   # padding rows stay zero
    params[wo.P_W2:wo.P_B2] = 0.1 * rng.standard_normal(2 * wo.HIDDEN * wo.HIDDEN)
    params[wo.P_B2:wo.P_W3] = 0.05 * rng.standard_normal(wo.HIDDEN)
    params[wo.P_W3:wo.P_B3] = 0.1 * rng.standard_normal(wo.HIDDEN)
    params[wo.P_B3] = 0.1
    r = 4
    cluster = rng.integers(0, r, n)
    B = 3
    sets = [rng.choice(n, size=k, replace=False) for k in (1, 3, 5)]
    pushes = [wo.push(n, g.row_ptr, g.col, cluster, r, s, 0.85) for s in sets]
    mix = np.stack([p[1] for p in pushes])
    tmass = np.array([p[2] for p in pushes])
    K = np.abs(rng.standard_normal((2 * r + 1, r)))
    tails = np.abs(rng.standard_normal((B, n))) * (0.5 / n)
    return g, x1, params, in_rp, in_col, cluster, r, mix, K, tmass, tails


def test_analytic_gradient_matches_finite_differences():
    g, x1, params, in_rp, in_col, cluster, r, mix, K, tmass, tails = small_case()
    args = (x1, in_rp, in_col, g.row_ptr, g.col, cluster, r, mix, K, tmass, tails)
    loss, grad = wo.loss_grad(params, *args, emulate_bf16=False)
    assert np.isfinite(loss) and loss > 0
    rng = np.random.default_rng(1)
    pick = np.concatenate([
        rng.choice(np.arange(wo.P_W1, wo.P_W1 + 36 * wo.HIDDEN), 12, replace=False),
        wo.P_W1 + 36 * wo.HIDDEN + rng.choice(wo.HIDDEN, 4, replace=False),   # layer-1 bias row
        rng.choice(np.arange(wo.P_W2, wo.P_B2), 12, replace=False),
        rng.choice(np.arange(wo.P_B2, wo.P_W3), 4, replace=False),
        rng.choice(np.arange(wo.P_W3, wo.P_B3), 6, replace=False),
        [wo.P_B3]])
    fd = wo.fd_grad(params, pick, 1e-6, *args, emulate_bf16=False)
    an = grad[pick]
    scale = np.abs(an).max()
    assert scale > 0
    assert np.abs(fd - an).max() <= 1e-4 * scale + 1e-9, np.c_[pick, fd, an]
    # padding rows of W1 get no gradient
    assert not grad[wo.P_W1 + 37 * wo.HIDDEN:wo.P_W2].any()


def test_push_matches_dense_series():
    g = gen.erdos_renyi(50, 0.06, 0.1, seed=3)
    n = g.n
    P = np.zeros((n, n))
    deg = np.diff(g.row_ptr)
    for u in range(n):
        for v in g.col[g.row_ptr[u]:g.row_ptr[u + 1]]:
            P[v, u] += 1.0 / deg[u]
    cluster = np.arange(n) % 5
    seeds = [4, 9, 9, 30]
    s = np.zeros(n)
    for u in seeds:
        s[u] += 0.25
    d = 0.85
    local, mix, tm, r1 = wo.push(n, g.row_ptr, g.col, cluster, 5, seeds, d)
    ser = (1 - d) * sum(d ** k * np.linalg.matrix_power(P, k) @ s for k in range(4))
    assert np.abs(local - ser).max() < 1e-15
    f3 = np.linalg.matrix_power(P, 3) @ s
    f4 = P @ f3
    assert np.allclose(mix[:5], np.bincount(cluster, weights=f3, minlength=5), atol=1e-15)
    assert np.allclose(mix[5:10], np.bincount(cluster, weights=f4, minlength=5), atol=1e-15)
    assert mix[10] == 1.0
    # tail mass: 1 minus the local mass; cold residual: one PPR step from s
    assert abs(tm - (1 - local.sum())) < 1e-14
    dang = deg == 0
    Fs = (1 - d) * s + d * (P @ s) + d * s[dang].sum() * s
    assert abs(r1 - np.abs(Fs - s).sum()) < 1e-14


def test_least_squares_fit():
    rng = np.random.default_rng(2)
    X = rng.standard_normal((200, 9))
    Kt = rng.standard_normal((9, 4))
    Y = X @ Kt
    K = wo.fit_coupling(X, Y, 1e-12)
    assert np.abs(K - Kt).max() < 1e-8


def test_bf16_rounding():
    a = np.array([1.0, 1.00390625, 1.005859375, -3.14159, 0.0, 65504.0])
    b = wo.bf16(a)
    assert b[0] == 1.0 and b[1] == 1.0  # halfway: ties to even
    assert b[2] == 1.0078125
    assert abs(b[3] + 3.140625) < 1e-12 and b[4] == 0.0
