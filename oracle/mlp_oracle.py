"""CPU restatement (numpy, FP64) of the learned per-pair M2L order selection:
the order model's forward pass, cross-entropy gradient, Adam update and order
decoding, and the per-pair features and training labels.

TEST INFRASTRUCTURE ONLY: imported by tests/ as the checker of the CUDA
kernels in fmmgen_gb300/csrc/learn.cu.  The product package never imports it.

The reference has no counterpart (its FMM applies one order to every M2L
pair: example/calculate.cpp:190-206), so parity here is against this
restatement of the method, whose M2L parts use the oracle's own fmmgen
operators (oracle/fmm_oracle.c or_M2L, fmmgen/expansions.py:144-172).
"""
import math

import numpy as np

NIN, NH, NOUT, QMIN = 16, 64, 11, 2
# parameter layout (FP32 on the device): W1[64][16], b1[64], W2[64][64], b2[64], W3[11][64], b3[11]
SHAPES = [("W1", (NH, NIN)), ("b1", (NH,)), ("W2", (NH, NH)), ("b2", (NH,)), ("W3", (NOUT, NH)), ("b3", (NOUT,))]
NPARAM = sum(int(np.prod(s)) for _, s in SHAPES)


def unpack(params):
    params = np.asarray(params, dtype=np.float64)
    out, o = {}, 0
    for name, shp in SHAPES:
        n = int(np.prod(shp))
        out[name] = params[o:o + n].reshape(shp)
        o += n
    return out


def pack(d):
    return np.concatenate([np.asarray(d[name], dtype=np.float64).ravel() for name, _ in SHAPES])


def forward(params, X):
    """Logits z [n][11] and the activations (h1, h2) of the ReLU layers."""
    P = unpack(params)
    X = np.asarray(X, dtype=np.float64)
    h1 = np.maximum(X @ P["W1"].T + P["b1"], 0.0)
    h2 = np.maximum(h1 @ P["W2"].T + P["b2"], 0.0)
    z = h2 @ P["W3"].T + P["b3"]
    return z, h1, h2


def softmax(z):
    e = np.exp(z - z.max(axis=1, keepdims=True))
    return e / e.sum(axis=1, keepdims=True)


def loss_grad(params, X, y):
    """Mean cross-entropy of the logits against labels y (0..10) and its gradient
    with respect to the flat parameter vector."""
    P = unpack(params)
    X = np.asarray(X, dtype=np.float64)
    y = np.asarray(y, dtype=np.int64)
    n = X.shape[0]
    z, h1, h2 = forward(params, X)
    zm = z.max(axis=1, keepdims=True)
    lse = np.log(np.exp(z - zm).sum(axis=1)) + zm[:, 0]
    loss = float(np.mean(lse - z[np.arange(n), y]))
    g3 = softmax(z)
    g3[np.arange(n), y] -= 1.0
    g3 /= n
    g2 = (g3 @ P["W3"]) * (h2 > 0)
    g1 = (g2 @ P["W2"]) * (h1 > 0)
    grad = {"W3": g3.T @ h2, "b3": g3.sum(0), "W2": g2.T @ h1, "b2": g2.sum(0), "W1": g1.T @ X, "b1": g1.sum(0)}
    return loss, pack(grad)


def adam(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step (step >= 1); returns new (params, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return params - lr * mh / (np.sqrt(vh) + eps), m, v


def predict(params, X, delta, qmax):
    """Lowest order q whose cumulative predicted probability P(q* <= q) reaches
    1 - delta, clamped to [2, qmax]; also returns that cumulative table."""
    z, _, _ = forward(params, X)
    cum = np.cumsum(softmax(z), axis=1)
    hit = cum >= 1.0 - delta
    first = np.where(hit.any(axis=1), hit.argmax(axis=1), NOUT - 1)
    return np.clip(first + QMIN, QMIN, qmax).astype(np.uint8), cum


# ---------------------------------------------------------------------------
# features and labels
# ---------------------------------------------------------------------------
def _nterms(p):
    return (p + 1) * (p + 2) * (p + 3) // 6 if p >= 0 else 0


def multi_indices(p):
    """fmmgen's degree-major multi-index order (fmmgen/utils.py Nterms layout)."""
    out = []
    for d in range(p + 1):
        for nx in range(d, -1, -1):
            for ny in range(d - nx, -1, -1):
                out.append((nx, ny, d - nx - ny))
    return out


def degree_norms(Mrow, order, so, s):
    """2-norm of each degree block of the scaled multipole M~_m = M_m / s^|m|
    (row starts at degree so), indexed 0..12."""
    mi = multi_indices(order)
    off = _nterms(so - 1)
    out = np.zeros(13)
    for d in range(so, order + 1):
        blk = np.array([Mrow[j - off] / s ** sum(mi[j]) for j in range(_nterms(d - 1), _nterms(d))])
        out[d] = math.sqrt(float(np.sum(blk * blk)))
    return out


def pair_features(mn, sep, dlev, wsum, etol):
    """Features of one pair (B -> A): mn = degree norms of B's scaled multipole,
    sep = |c_A - c_B| / s_A, dlev = l_B - l_A; wsum = the target's summed
    estimates (from pair_estimate); etol = eps T_A, the pair's error budget."""
    w, part = pair_estimate(mn, sep, dlev)
    f = np.zeros(NIN)
    f[0] = dlev
    f[1] = math.log2(sep)
    f[2] = math.log10(max(w / max(wsum, 1e-30), 1e-30))
    for d in range(1, 13):
        f[2 + d] = math.log10(max(part[d] / max(w, 1e-30), 1e-30))
    f[15] = math.log10(max(w / (sep * etol), 1e-30))
    return f


def pair_estimate(mn, sep, dlev):
    """Estimated far field of the pair at the target, sum_d rho^d |M~_d| / sep^(d+1),
    rho = s_B / s_A = 2^-dlev, and its per-degree parts."""
    rho = 2.0 ** (-dlev)
    part = np.array([mn[d] * rho ** d / sep ** (d + 1) for d in range(13)])
    return float(part.sum()), part


def grad_bound_table(p):
    """g_n = max over the cell box |y_i| <= 1 of |grad (y^n / n!)|, |n| <= p."""
    f = math.factorial
    g = []
    for n in multi_indices(p):
        s = 0.0
        for a in range(3):
            if n[a] == 0:
                continue
            den = 1.0
            for b in range(3):
                den *= f(n[b] - (1 if a == b else 0))
            s += 1.0 / (den * den)
        g.append(math.sqrt(s))
    return np.array(g)


def truncation_bounds(m2l, dvec, Mrow, order, so, sA):
    """err_q, q = 0..order, for one pair: sum_n g_n s_A^(|n|+1) |L_p[n] - L_q[n]|
    where L_q is fmmgen's order-q M2L of the source multipole (unscaled) across
    dvec = c_A - c_B; m2l(x, y, z, M, L, order, so) is that operator."""
    ls = _nterms(order - so)
    mi = multi_indices(order)
    g = grad_bound_table(order)[:ls]
    scale = np.array([sA ** (sum(mi[i]) + 1) for i in range(ls)])
    Lp = np.zeros(ls)
    m2l(dvec[0], dvec[1], dvec[2], Mrow, Lp, order, so)
    err = np.zeros(order + 1)
    for q in range(so + 1, order):
        Lq = np.zeros(ls)
        m2l(dvec[0], dvec[1], dvec[2], Mrow, Lq, q, so)
        err[q] = float(np.sum(g * scale * np.abs(Lp - Lq)))
    err[:so + 1] = np.inf
    return err


def label_from_bounds(err, order, tol):
    """Lowest q >= 2 whose bound is within tol; order when none is; label q - 2."""
    for q in range(QMIN, order):
        if err[q] <= tol:
            return q - QMIN
    return order - QMIN


def near_field(pos, q, leaves, p2p):
    """The P2P part of the Coulomb field: for every (target leaf, source leaf)
    pair, E_i += sum_j q_j (x_i - x_j) / |x_i - x_j|^3, j != i; leaves maps a
    cell id to its particle indices."""
    E = np.zeros((len(pos), 3))
    for a, b in p2p:
        ia, ib = leaves[int(a)], leaves[int(b)]
        r = pos[ia][:, None, :] - pos[ib][None, :, :]
        d2 = np.sum(r * r, axis=2)
        same = ia[:, None] == ib[None, :]
        d2[same] = 1.0
        w = q[ib][None, :] / (d2 * np.sqrt(d2))
        w[same] = 0.0
        E[ia] += np.einsum("ij,ijk->ik", w, r)
    return E


def tol_scale(Enear, npairs):
    """sqrt(sum_i |E_near,i|^2 / P): the system's share of the squared error
    budget per M2L pair."""
    return math.sqrt(float(np.sum(Enear * Enear)) / max(npairs, 1))


def cell_tol(tscale, s, n):
    """T_A = tscale s_A^2 / sqrt(n_A): pair budget over eps in A's scaled units."""
    return tscale * s * s / math.sqrt(max(n, 1))


def pair_terms(q, so):
    """Multiply-adds of one M2L pair at order q: pairs (n, m), |m| >= so, |n| + |m| <= q."""
    return sum((d + 1) * (d + 2) // 2 * _nterms(q - d) for d in range(so, q + 1))
