"""CPU oracle of the learned warm start (test infrastructure only).

The reference crate has no warm start; this module restates, in FP64 numpy,
the exact arithmetic the library's warm start defines (include/gops.h,
gops_warm_*), so that the device kernels can be checked against it:

* ``push``          the exact local terms (1-d)(s + d P s + d^2 P^2 s + d^3 P^3 s),
                    the cluster mixes of P^3 s and P^4 s, the tail mass and the
                    cold first-step residual ||F(s) - s||_1 of personalized
                    PageRank (src/ppr.rs:90-156 for F: teleport to s,
                    dangling mass back to s);
* ``forward``       the two-layer message-passing network w = exp(MPNN(x1)),
                    optionally emulating the device's BF16 roundings;
* ``loss_grad``     the L1 tail loss and its analytic gradient;
* ``fd_grad``       central finite differences of ``loss_grad``'s loss;
* ``fit_coupling``  the ridge least-squares fit of the cluster coupling K.

Only tests/ (and smoke checks) import this module; the library never does.
"""
from __future__ import annotations

import numpy as np

W_IN, HIDDEN, FEAT = 48, 128, 18
P_W1 = 0
P_W2 = P_W1 + W_IN * HIDDEN
P_B2 = P_W2 + 2 * HIDDEN * HIDDEN
P_W3 = P_B2 + HIDDEN
P_B3 = P_W3 + HIDDEN
P_COUNT = P_B3 + 1
U_CLAMP = 20.0


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def in_csr(n, row_ptr, col):
    """In-edge CSR in original order: row v lists the sources of edges into
    v in ascending source order (a stable sort by destination)."""
    row_ptr = np.asarray(row_ptr, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    src = np.repeat(np.arange(n, dtype=np.int64), np.diff(row_ptr))
    order = np.argsort(col, kind="stable")
    in_col = src[order]
    in_rp = np.zeros(n + 1, dtype=np.int64)
    np.add.at(in_rp, col + 1, 1)
    return np.cumsum(in_rp), in_col


def push(n, row_ptr, col, cluster, r, seeds, d):
    """(local[n], mix[2r+1], tail_mass, r1_cold) of one seed set (FP64)."""
    row_ptr = np.asarray(row_ptr, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    cluster = np.asarray(cluster, dtype=np.int64)
    deg = np.diff(row_ptr).astype(np.float64)
    inv = np.where(deg > 0, 1.0 / np.maximum(deg, 1.0), 0.0)
    src = np.repeat(np.arange(n), np.diff(row_ptr))
    seeds = np.asarray(seeds, dtype=np.int64)
    s = np.zeros(n)
    np.add.at(s, seeds, 1.0 / len(seeds))

    def step(x):  # P x: mass of x moved along out-edges (dangling mass dropped)
        y = np.zeros(n)
        np.add.at(y, col, (x * inv)[src])
        return y

    f1 = step(s)
    f2 = step(f1)
    f3 = step(f2)
    f4 = step(f3)
    local = (1 - d) * (s + d * f1 + d * d * f2 + d ** 3 * f3)
    h3 = np.bincount(cluster, weights=f3, minlength=r)
    h4 = np.bincount(cluster, weights=f4, minlength=r)
    mix = np.concatenate([h3, h4, [1.0]])
    m1, m2, m3 = f1.sum(), f2.sum(), f3.sum()
    tail_mass = 1.0 - (1 - d) * (1 + d * m1 + d * d * m2 + d ** 3 * m3)
    r1 = d * np.abs(f1 - m1 * s).sum()
    return local, mix, tail_mass, r1


def push_many(n, row_ptr, col, cluster, r, seed_ptr, seed_idx, d):
    """push() for many sets at once (scipy sparse products): local [B, n],
    mix [B, 2r+1], tail_mass [B]."""
    import scipy.sparse as sp
    row_ptr = np.asarray(row_ptr, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    deg = np.diff(row_ptr).astype(np.float64)
    src = np.repeat(np.arange(n), np.diff(row_ptr))
    P = sp.csr_matrix((1.0 / deg[src], (col, src)), shape=(n, n))
    B = len(seed_ptr) - 1
    rows, cols, vals = [], [], []
    for j in range(B):
        k = seed_idx[seed_ptr[j]:seed_ptr[j + 1]]
        rows.append(np.asarray(k, dtype=np.int64))
        cols.append(np.full(len(k), j))
        vals.append(np.full(len(k), 1.0 / len(k)))
    S = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))), shape=(n, B))
    S = np.asarray(S.todense())
    f1 = P @ S
    f2 = P @ f1
    f3 = P @ f2
    f4 = P @ f3
    local = ((1 - d) * (S + d * f1 + d * d * f2 + d ** 3 * f3)).T
    H = sp.csr_matrix((np.ones(n), (np.arange(n), np.asarray(cluster, dtype=np.int64))), shape=(n, r))
    mix = np.c_[(H.T @ f3).T, (H.T @ f4).T, np.ones(B)]
    tm = 1.0 - (1 - d) * (1 + d * f1.sum(0) + d * d * f2.sum(0) + d ** 3 * f3.sum(0))
    return local, mix, tm


def forward(x1, params, in_rp, in_col, emulate_bf16=True):
    """w = exp(clamp(u)) of the network and the activations backward needs."""
    rnd = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    n = x1.shape[0]
    W1 = rnd(params[P_W1:P_W2].reshape(W_IN, HIDDEN))
    W2 = rnd(params[P_W2:P_B2].reshape(2 * HIDDEN, HIDDEN))
    b2 = params[P_B2:P_W3].astype(np.float64)
    w3 = params[P_W3:P_B3].astype(np.float64)
    b3 = float(params[P_B3])
    X = np.asarray(x1, dtype=np.float64)
    H1 = rnd(np.maximum(X @ W1, 0.0))
    indeg = np.diff(in_rp)
    dst = np.repeat(np.arange(n), indeg)
    agg = np.zeros((n, HIDDEN))
    np.add.at(agg, dst, H1[in_col])
    inv_in = np.where(indeg > 0, 1.0 / np.maximum(indeg, 1), 0.0)
    A1 = rnd(agg * inv_in[:, None])
    Z = np.concatenate([H1, A1], 1)
    H2 = rnd(np.maximum(Z @ W2 + b2, 0.0))
    u = H2 @ w3 + b3
    uc = np.clip(u, -U_CLAMP, U_CLAMP)
    w = np.exp(uc)
    cache = dict(X=X, W1=W1, W2=W2, w3=w3, H1=H1, A1=A1, Z=Z, H2=H2, u=u, inv_in=inv_in, dst=dst,
                 clamped=np.abs(u) >= U_CLAMP)
    return w, cache


def coefficients(mix, K, tmass, w, cluster, r):
    """coef[j][c] = tm_j m_jc / (sum_c m_jc * cw_c), m = relu(mix_j K)."""
    cw = np.bincount(cluster, weights=w, minlength=r)
    m = np.maximum(np.asarray(mix, dtype=np.float64) @ np.asarray(K, dtype=np.float64), 0.0)
    tot = m.sum(1, keepdims=True)
    with np.errstate(divide="ignore", invalid="ignore"):
        coef = np.where((tot > 0) & (cw[None] > 0), tmass[:, None] * m / (tot * cw[None]), 0.0)
    return coef, cw


def loss_grad(params, x1, in_rp, in_col, out_rp, out_col, cluster, r, mix, K, tmass, tails,
              emulate_bf16=True):
    """Mean over sets of ||w_i coef[j][a_i] - tail_j||_1 and its gradient."""
    rnd = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    cluster = np.asarray(cluster, dtype=np.int64)
    w, c = forward(x1, params, in_rp, in_col, emulate_bf16)
    coef, cw = coefficients(mix, K, tmass, w, cluster, r)
    B = tails.shape[0]
    pred = w[None, :] * coef[:, cluster]
    e = pred - tails
    loss = np.abs(e).sum() / B
    g = np.sign(e)
    t1 = (g * coef[:, cluster]).sum(0)
    S = np.stack([np.bincount(cluster, weights=g[j] * w, minlength=r) for j in range(B)])
    with np.errstate(divide="ignore", invalid="ignore"):
        s_term = np.where(cw[None] > 0, coef * S / cw[None], 0.0)
    dw = t1 - s_term[:, cluster].sum(0)
    du = np.where(c["clamped"], 0.0, dw * w / B)
    grad = np.zeros(P_COUNT)
    gv = du[:, None] * c["w3"][None, :] * (c["H2"] > 0)
    grad[P_W3:P_B3] = du @ c["H2"]
    grad[P_B3] = du.sum()
    grad[P_B2:P_W3] = gv.sum(0)
    G2 = rnd(gv)
    grad[P_W2:P_B2] = (c["Z"].T @ G2).ravel()
    GX = rnd(G2 @ c["W2"].T)
    n = x1.shape[0]
    out_rp = np.asarray(out_rp, dtype=np.int64)
    out_col = np.asarray(out_col, dtype=np.int64)
    src = np.repeat(np.arange(n), np.diff(out_rp))
    back = np.zeros((n, HIDDEN))
    np.add.at(back, src, GX[out_col, HIDDEN:] * c["inv_in"][out_col][:, None])
    G1 = rnd((GX[:, :HIDDEN] + back) * (c["H1"] > 0))
    grad[P_W1:P_W2] = (c["X"].T @ G1).ravel()
    return loss, grad


def fd_grad(params, idx, h, *args, **kw):
    """Central differences of loss_grad's loss at the parameters `idx`."""
    out = np.zeros(len(idx))
    for q, i in enumerate(idx):
        p1 = params.copy()
        p1[i] += h
        p0 = params.copy()
        p0[i] -= h
        out[q] = (loss_grad(p1, *args, **kw)[0] - loss_grad(p0, *args, **kw)[0]) / (2 * h)
    return out


def fit_coupling(mix, ymass, ridge):
    """K = (X^T X + lambda I)^-1 X^T Y with lambda = ridge * trace / dim."""
    X = np.asarray(mix, dtype=np.float64)
    G = X.T @ X
    lam = ridge * (np.trace(G) / G.shape[0] if np.trace(G) > 0 else 1.0)
    return np.linalg.solve(G + lam * np.eye(G.shape[0]), X.T @ np.asarray(ymass, dtype=np.float64))


def code(n, row_ptr, col, z0, steps):
    """The random-projection code: z0 diffused `steps` times by
    (mean over in-neighbours + mean over out-neighbours) / 2, each column
    standardised after every step."""
    row_ptr = np.asarray(row_ptr, dtype=np.int64)
    col = np.asarray(col, dtype=np.int64)
    src = np.repeat(np.arange(n), np.diff(row_ptr))
    dout = np.diff(row_ptr).astype(np.float64)
    din = np.bincount(col, minlength=n).astype(np.float64)
    z = np.asarray(z0, dtype=np.float64).copy()
    for _ in range(steps):
        a = np.zeros_like(z)
        np.add.at(a, col, z[src])
        b = np.zeros_like(z)
        np.add.at(b, src, z[col])
        a = a * np.where(din > 0, 1.0 / np.maximum(din, 1), 0.0)[:, None]
        b = b * np.where(dout > 0, 1.0 / np.maximum(dout, 1), 0.0)[:, None]
        z = 0.5 * (a + b)
        sd = z.std(0)
        z = (z - z.mean(0)) / np.where(sd > 1e-15, sd, 1.0)
    return z


def splitmix64(z):
    z = (int(z) + 0x9E3779B97F4A7C15) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & 0xFFFFFFFFFFFFFFFF
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & 0xFFFFFFFFFFFFFFFF
    return z ^ (z >> 31)


def code_init(n, seed):
    """The code's starting Gaussian matrix (n x 16): two 24-bit uniforms per
    entry from SplitMix64 of (seed, index), Box-Muller transform."""
    s = splitmix64(seed)
    out = np.empty(n * 16)
    for i in range(n * 16):
        h = splitmix64(s ^ splitmix64(i))
        u1 = ((h >> 40) + 1) / 16777216.0
        u2 = ((h >> 16) & 0xFFFFFF) / 16777216.0
        out[i] = np.sqrt(-2.0 * np.log(u1)) * np.cos(2 * np.pi * u2)
    return out.reshape(n, 16)
