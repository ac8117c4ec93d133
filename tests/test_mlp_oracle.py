"""CPU checks of the learned-order oracle (oracle/mlp_oracle.py) and the
host-side pieces of fmmgen_gb300.learned: the oracle's gradient against finite
differences, Adam and order decoding by hand, the truncation bounds against
their definition, work counts against brute-force enumeration, and the
first-layer normalisation fold."""
import math

import numpy as np
import pytest

from oracle import mlp_oracle as mo


def rand_model(seed, n=64):
    rng = np.random.default_rng(seed)
    params = rng.standard_normal(mo.NPARAM) * 0.3
    X = rng.standard_normal((n, mo.NIN))
    y = rng.integers(0, mo.NOUT, n)
    return params, X, y


def test_layout():
    assert mo.NPARAM == 64 * 16 + 64 + 64 * 64 + 64 + 11 * 64 + 11 == 5963
    p = np.arange(mo.NPARAM, dtype=np.float64)
    assert np.array_equal(mo.pack(mo.unpack(p)), p)
    assert mo.unpack(p)["b3"][0] == mo.NPARAM - 11


def test_gradient_matches_finite_differences():
    params, X, y = rand_model(1)
    loss, g = mo.loss_grad(params, X, y)
    rng = np.random.default_rng(2)
    # every bias and a sample of weights of every layer
    idx = list(range(1024, 1088)) + list(range(5184, 5248)) + list(range(5952, 5963))
    idx += list(rng.choice(1024, 40, replace=False)) + list(1088 + rng.choice(4096, 40, replace=False))
    idx += list(5248 + rng.choice(704, 40, replace=False))
    h = 1e-6
    for i in idx:
        e = np.zeros(mo.NPARAM)
        e[i] = h
        num = (mo.loss_grad(params + e, X, y)[0] - mo.loss_grad(params - e, X, y)[0]) / (2 * h)
        assert abs(num - g[i]) <= 1e-6 + 1e-5 * abs(g[i]), (i, num, g[i])
    assert loss > 0


def test_loss_is_cross_entropy():
    params, X, y = rand_model(3, 10)
    z, _, _ = mo.forward(params, X)
    ref = np.mean([-math.log(math.exp(z[k, y[k]]) / np.exp(z[k]).sum()) for k in range(10)])
    assert abs(mo.loss_grad(params, X, y)[0] - ref) < 1e-12


def test_adam_by_hand():
    rng = np.random.default_rng(4)
    p, g = rng.standard_normal(5), rng.standard_normal(5)
    m, v = np.zeros(5), np.zeros(5)
    p1, m1, v1 = mo.adam(p, g, m, v, 1, 0.01)
    # first bias-corrected step moves every parameter by lr against the sign of its gradient
    assert np.allclose(p1, p - 0.01 * g / (np.abs(g) + 1e-8))
    p2, _, _ = mo.adam(p1, g, m1, v1, 2, 0.01)
    assert np.allclose(p2, p1 - 0.01 * g / (np.abs(g) + 1e-8), atol=1e-12)


def test_predict_decoding():
    params, X, _ = rand_model(5, 200)
    q0, cum = mo.predict(params, X, 0.0, 12)
    assert np.all(cum[:, -1] > 0.999999)
    for d in (0.01, 0.1, 0.5):
        q, _ = mo.predict(params, X, d, 12)
        assert np.all(q <= q0)  # a larger delta never raises an order
        for k in range(0, 200, 17):  # the lowest order whose cumulative reaches 1 - delta
            first = int(np.argmax(cum[k] >= 1 - d))
            assert q[k] == first + 2
    q, _ = mo.predict(params, X, 0.0, 7)
    assert q.max() <= 7 and q.min() >= 2


def test_pair_terms_brute_force():
    from fmmgen_gb300.learned import pair_terms

    for so in (0, 1):
        for q in range(so + 1, 13):
            mi = mo.multi_indices(q)
            brute = sum(1 for n in mi for m in mi if sum(m) >= so and sum(n) + sum(m) <= q)
            assert mo.pair_terms(q, so) == brute == pair_terms(q, so)


def test_multi_index_order_matches_oracle(oracle_lib):
    mi = mo.multi_indices(12)
    for i, (x, y, z) in enumerate(mi):
        assert oracle_lib.lib().or_index(x, y, z) == i


def test_grad_bound_table():
    g = mo.grad_bound_table(4)
    mi = mo.multi_indices(4)
    assert g[0] == 0.0
    # n = (2, 0, 0): grad (x^2 / 2) = (x, 0, 0), max 1 on the box
    assert g[mi.index((2, 0, 0))] == 1.0
    # n = (1, 1, 0): grad (x y) = (y, x, 0), max sqrt(2)
    assert abs(g[mi.index((1, 1, 0))] - math.sqrt(2)) < 1e-15
    # brute force over the box corners (the maximum of |monomial derivative| sits there)
    corners = [np.array(c, float) for c in np.ndindex(2, 2, 2)]
    for n in mi[1:]:
        best = 0.0
        for c in corners:
            y = 2 * c - 1
            gr = []
            for a in range(3):
                if n[a] == 0:
                    gr.append(0.0)
                    continue
                e = list(n)
                e[a] -= 1
                gr.append(np.prod([y[b] ** e[b] / math.factorial(e[b]) for b in range(3)]))
            best = max(best, float(np.linalg.norm(gr)))
        assert abs(best - g[mi.index(n)]) < 1e-14


def test_truncation_bounds_definition(oracle_lib):
    rng = np.random.default_rng(6)
    order, so = 8, 0
    ms = oracle_lib.msize(order, so)
    M = rng.standard_normal(ms) * np.array([0.3 ** sum(m) for m in mo.multi_indices(order)])
    d = np.array([2.1, -0.7, 1.3])
    err = mo.truncation_bounds(oracle_lib.M2L, d, M, order, so, 0.5)
    assert np.isinf(err[0])
    assert np.all(np.diff(err[1:order]) < 0)  # well separated: higher orders drop less
    # the bound at q against the terms of total degree > q computed directly
    D = oracle_lib.derivs(*d, order)
    mi = mo.multi_indices(order)
    g = mo.grad_bound_table(order)
    q = 4
    tot = 0.0
    for i, n in enumerate(mi):
        s = sum(D[oracle_lib.lib().or_index(n[0] + m[0], n[1] + m[1], n[2] + m[2])] * M[j]
                for j, m in enumerate(mi) if sum(n) + sum(m) <= order and sum(n) + sum(m) > q)
        tot += g[i] * 0.5 ** (sum(n) + 1) * abs(s)
    assert abs(tot - err[q]) <= 1e-12 * abs(tot)
    assert mo.label_from_bounds(err, order, err[5] * 1.0000001) == 5 - 2
    assert mo.label_from_bounds(err, order, 0.0) == order - 2


def test_fold_normalisation():
    from fmmgen_gb300.learned import fold_normalisation, init_params

    rng = np.random.default_rng(7)
    p = init_params(3).astype(np.float64)
    X = rng.standard_normal((50, 16)) * 5 + 3
    mean, std = X.mean(0), X.std(0)
    z0, _, _ = mo.forward(p, (X - mean) / std)
    z1, _, _ = mo.forward(fold_normalisation(p, mean, std).astype(np.float64), X)
    assert np.allclose(z0, z1, rtol=1e-4, atol=1e-4)
