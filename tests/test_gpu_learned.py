"""Learned per-pair M2L orders on the GPU: the order-model kernels (inference,
training step, Adam) against the FP64 numpy oracle, features and labels
against their CPU restatement, the variable-order M2L pass against the
oracle's FMM with the same per-pair orders, and what the trained model gains
over the fixed-order FMM at the same error."""
import os

import numpy as np
import pytest
import torch

from oracle import mlp_oracle as mo

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def rand_inputs(seed, n):
    rng = np.random.default_rng(seed)
    params = (rng.standard_normal(mo.NPARAM) * 0.2).astype(np.float32)
    X = (rng.standard_normal((n, mo.NIN)) * 2).astype(np.float32)
    y = rng.integers(0, mo.NOUT, n).astype(np.uint8)
    return params, X, y


def cuda(a):
    return torch.tensor(a, device="cuda")


# ---------------------------------------------------------------------------
# order-model kernels vs the oracle
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("n", [1, 37, 3000])
def test_train_step_matches_oracle(fg, n):
    from fmmgen_gb300 import learned

    params, X, y = rand_inputs(10 + n, n)
    grad = torch.full((mo.NPARAM,), 7.0, device="cuda")  # overwritten, not accumulated
    loss = torch.full((1,), 0.5, device="cuda")          # incremented
    learned.train_step(cuda(params), cuda(X), cuda(y), grad, loss)
    torch.cuda.synchronize()
    lo, go = mo.loss_grad(params.astype(np.float64), X.astype(np.float64), y)
    g = grad.cpu().numpy().astype(np.float64)
    assert abs(float(loss.item()) - 0.5 - lo) <= 1e-5 * max(1.0, abs(lo))
    scale = np.abs(go).max()
    assert np.all(np.abs(g - go) <= 1e-5 * scale + 1e-3 * np.abs(go)), np.abs(g - go).max() / scale


def test_adam_matches_oracle(fg):
    from fmmgen_gb300 import learned

    rng = np.random.default_rng(20)
    p, g, m = (rng.standard_normal(mo.NPARAM).astype(np.float32) for _ in range(3))
    v = np.abs(rng.standard_normal(mo.NPARAM)).astype(np.float32)
    P, M, V = cuda(p), cuda(m), cuda(v)
    learned.adam_step(P, cuda(g), M, V, 3, 1e-2)
    po, mo_, vo = mo.adam(p.astype(np.float64), g.astype(np.float64), m.astype(np.float64), v.astype(np.float64),
                          3, 1e-2)
    assert np.allclose(P.cpu().numpy(), po, rtol=1e-5, atol=1e-6)
    assert np.allclose(M.cpu().numpy(), mo_, rtol=1e-5, atol=1e-7)
    assert np.allclose(V.cpu().numpy(), vo, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("delta,qmax", [(0.0, 12), (0.05, 12), (0.3, 9)])
def test_predict_matches_oracle(fg, delta, qmax):
    from fmmgen_gb300 import learned

    params, X, _ = rand_inputs(30, 20000)
    q = learned.predict(cuda(params), cuda(X), delta, qmax).cpu().numpy()
    qo, cum = mo.predict(params.astype(np.float64), X.astype(np.float64), delta, qmax)
    bad = np.nonzero(q != qo)[0]
    # a row may only differ where a cumulative probability sits at the threshold
    for k in bad:
        assert np.min(np.abs(cum[k] - (1 - delta))) < 1e-5, (k, q[k], qo[k])
    assert len(bad) <= 5
    assert q.min() >= 2 and q.max() <= qmax


def test_training_reduces_loss(fg):
    """The model trains on the GPU with the project's own kernels: minibatch
    Adam on pairs of a small fixed-order FMM lowers the cross-entropy, and the
    trained model predicts the labels far better than the most common one."""
    from fmmgen_gb300 import learned

    n = 20000
    rng = np.random.default_rng(40)
    pos = learned.mixture_positions(n, nclusters=16, sigma=0.02, seed=40)
    t = fg.build_tree(pos, rng.uniform(-1, 1, (n, 1)), n, 64, 10, 0.5)
    X, y = learned.training_pairs(t, 1e-6)
    assert X.shape == (t.nm2l, 16) and y.shape == (t.nm2l,)
    yh = y.cpu().numpy()
    assert yh.max() <= 8 and yh.min() >= 0  # orders 2..10
    assert len(np.unique(yh)) >= 5
    model = learned.OrderModel(seed=1)
    hist = model.fit(X, y, steps=400, batch=4096, lr=3e-3, lr_final=3e-4)
    assert hist[-1] < 0.7 * hist[0], hist
    # accuracy of the most probable order against the labels
    z = mo.forward(model.params.cpu().numpy().astype(np.float64), X.cpu().numpy().astype(np.float64))[0]
    acc = float(np.mean(np.argmax(z, axis=1) == yh))
    major = float(np.bincount(yh).max() / len(yh))
    assert acc > major + 0.05, (acc, major)


# ---------------------------------------------------------------------------
# features and labels vs the restatement
# ---------------------------------------------------------------------------
def small_system(seed, n, p, ncrit=32):
    from fmmgen_gb300 import learned

    rng = np.random.default_rng(seed)
    pos = learned.mixture_positions(n, nclusters=8, sigma=0.03, seed=seed)
    S = rng.uniform(-1, 1, (n, 1))
    return pos, S


def oracle_view(fg, oracle_lib, pos, S, ncrit, p):
    """GPU tree, oracle tree, oracle cells, cell id -> oracle cell index."""
    t = fg.build_tree(torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda"), len(pos), ncrit, p, 0.5)
    ot = oracle_lib.OracleTree(pos, S, ncrit, p, 0.5, 0)
    oc = ot.cells()
    om = {int(i): k for k, i in enumerate(oc["id"])}
    return t, ot, oc, om


def budget_scale(t, pos, S):
    """The pair budget scale sqrt(sum |E_near|^2 / P) restated from the tree's
    leaves and P2P list."""
    c = t.cells()
    leaf_ids = c["id"][c["count"] < t.ncrit]
    leaves = {int(i): c["leaf_idx"][c["leaf_off"][k]:c["leaf_off"][k + 1]] for k, i in enumerate(leaf_ids)}
    _, p2p = t.lists()
    return mo.tol_scale(mo.near_field(pos, S[:, 0], leaves, p2p), t.nm2l)


def test_features_match_restatement(fg, oracle_lib):
    from fmmgen_gb300 import learned

    p, ncrit = 9, 32
    pos, S = small_system(50, 6000, p)
    t, ot, oc, om = oracle_view(fg, oracle_lib, pos, S, ncrit, p)
    eps = 1e-6
    t.compute_field_fmm(precision="fp64")
    feat = learned.order_features(t, eps).cpu().numpy()
    _, _, Mo, _ = ot.evaluate(want_ML=True)
    r0 = t.root()[3]
    pairs, _ = t.lists()
    ts = budget_scale(t, pos, S)
    norms = {}

    def mnorm(c):
        if c not in norms:
            k = om[c]
            norms[c] = mo.degree_norms(Mo[k], p, 0, r0 / 2.0 ** oc["level"][k])
        return norms[c]

    est = []
    for b, a in pairs:
        kb, ka = om[int(b)], om[int(a)]
        sA = r0 / 2.0 ** oc["level"][ka]
        sep = float(np.linalg.norm(oc["centre"][ka] - oc["centre"][kb])) / sA
        est.append((int(a), mnorm(int(b)), sep, int(oc["level"][kb] - oc["level"][ka])))
    wsum = {}
    for a, mn, sep, dl in est:
        wsum[a] = wsum.get(a, 0.0) + mo.pair_estimate(mn, sep, dl)[0]
    etol = {}
    for a, _, _, _ in est:
        if a not in etol:
            ka = om[a]
            etol[a] = eps * mo.cell_tol(ts, r0 / 2.0 ** oc["level"][ka], oc["nleaf"][ka])
    ref = np.array([mo.pair_features(mn, sep, dl, wsum[a], etol[a]) for a, mn, sep, dl in est])
    assert np.array_equal(feat[:, 0], ref[:, 0])
    assert np.abs(feat[:, 1] - ref[:, 1]).max() < 1e-5
    assert np.abs(feat[:, 2:] - ref[:, 2:]).max() < 2e-4


def test_labels_match_restatement(fg, oracle_lib):
    from fmmgen_gb300 import learned

    p, ncrit, eps = 10, 32, 1e-6
    pos, S = small_system(60, 5000, p)
    t, ot, oc, om = oracle_view(fg, oracle_lib, pos, S, ncrit, p)
    t.compute_field_fmm(precision="fp64")
    lab, errq = learned.order_labels(t, eps, errq=True)
    lab, errq = lab.cpu().numpy(), errq.cpu().numpy()
    _, _, Mo, _ = ot.evaluate(want_ML=True)
    r0 = t.root()[3]
    pairs, _ = t.lists()
    ts = budget_scale(t, pos, S)
    checked = 0
    for k in range(0, len(pairs), max(1, len(pairs) // 150)):
        b, a = int(pairs[k][0]), int(pairs[k][1])
        kb, ka = om[b], om[a]
        sA = r0 / 2.0 ** oc["level"][ka]
        cA = oc["centre"][ka]
        tol = eps * mo.cell_tol(ts, sA, oc["nleaf"][ka])
        err = mo.truncation_bounds(oracle_lib.M2L, cA - oc["centre"][kb], Mo[kb], p, 0, sA)
        ratio = err[2:p] / tol
        assert np.allclose(errq[k, : p - 2], ratio, rtol=1e-4, atol=1e-7), (k, errq[k, : p - 2], ratio)
        q = mo.label_from_bounds(err, p, tol)
        if not np.any(np.abs(ratio - 1) < 1e-4):
            assert lab[k] == q
        checked += 1
    assert checked >= 100


# ---------------------------------------------------------------------------
# the variable-order M2L pass
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("precision,tol", [("fp64", 1e-13), ("mixed", 2e-6)])
def test_all_orders_p_is_fixed_order(fg, precision, tol):
    rng = np.random.default_rng(70)
    n = 30000
    pos = torch.tensor(rng.uniform(0, 1, (n, 3)), device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (n, 1)), device="cuda")
    t = fg.build_tree(pos, S, n, 64, 8, 0.5)
    ref = t.compute_field_fmm(precision=precision).cpu().numpy()
    t.set_m2l_orders(np.full(t.nm2l, 8, np.uint8))
    F = t.compute_field_fmm(precision=precision).cpu().numpy()
    assert rel(F, ref) < tol
    assert np.all(t.m2l_orders() == 8)
    t.set_m2l_orders(None)
    assert np.array_equal(t.compute_field_fmm(precision=precision).cpu().numpy(), ref)


@pytest.mark.parametrize("so,p", [(0, 8), (1, 6), (0, 12)])
def test_var_orders_match_oracle(fg, oracle_lib, so, p):
    rng = np.random.default_rng(80 + p)
    n = 6000
    pos = rng.uniform(0, 1, (n, 3))
    S = rng.uniform(-1, 1, (n, 1)) if so == 0 else rng.standard_normal((n, 3))
    t = fg.build_tree(torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda"), n, 32, p, 0.5,
                      source_order=so)
    ot = oracle_lib.OracleTree(pos, S, 32, p, 0.5, so)
    pairs, _ = t.lists()
    orders = rng.integers(0, p + 3, t.nm2l).astype(np.uint8)  # clamped to [so + 1, p]
    t.set_m2l_orders(orders)
    F = t.compute_field_fmm(precision="fp64").cpu().numpy()
    used = t.m2l_orders()
    assert np.array_equal(used, np.clip(orders, so + 1, p))
    opairs, _ = ot.lists()
    where = {(int(b), int(a)): k for k, (b, a) in enumerate(pairs)}
    ot.set_m2l_orders(np.array([used[where[(int(b), int(a))]] for b, a in opairs], np.uint8))
    Fo, _ = ot.evaluate()
    assert rel(F, Fo) < 1e-12
    # and the truncation is real: the fixed-order field differs
    ot.set_m2l_orders(None)
    Ff, _ = ot.evaluate()
    assert rel(Ff, Fo) > 1e-9


def test_model_orders_are_predictions(fg):
    """With a model attached every pass predicts from its own multipoles: the
    orders it used are the model's predictions on that pass's features, and
    the field equals the pass with those orders given explicitly."""
    from fmmgen_gb300 import learned

    rng = np.random.default_rng(90)
    n = 40000
    pos = torch.tensor(learned.mixture_positions(n, seed=90), device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (n, 1)), device="cuda")
    t = fg.build_tree(pos, S, n, 64, 10, 0.5)
    model = learned.OrderModel(seed=3)
    for prec in ("fp64", "mixed"):
        model.attach(t, 0.1)
        F = t.compute_field_fmm(precision=prec).cpu().numpy()
        used = t.m2l_orders()
        pred = model.predict(learned.order_features(t), 0.1, qmax=10).cpu().numpy()
        assert np.array_equal(used, pred)
        assert len(np.unique(used)) > 1
        t.set_order_model(None)
        t.set_m2l_orders(used)
        assert np.array_equal(t.compute_field_fmm(precision=prec).cpu().numpy(), F)
        t.set_m2l_orders(None)


def test_orders_follow_the_build(fg):
    rng = np.random.default_rng(91)
    n = 20000
    pos = torch.tensor(rng.uniform(0, 1, (n, 3)), device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (n, 1)), device="cuda")
    t = fg.build_tree(pos, S, n, 64, 8, 0.5)
    t.set_m2l_orders(np.full(t.nm2l, 5, np.uint8))
    t.compute_field_fmm(precision="mixed")
    t.rebuild(torch.tensor(rng.uniform(0, 1, (n, 3)), device="cuda"))
    with pytest.raises(fg.FMMError):  # orders of the old lists
        t.compute_field_fmm(precision="mixed")
    with pytest.raises(ValueError):
        t.set_m2l_orders(np.full(t.nm2l + 1, 5, np.uint8))
    t.set_m2l_orders(None)
    t.compute_field_fmm(precision="mixed")


def test_model_under_graph_replay(fg):
    from fmmgen_gb300 import learned

    rng = np.random.default_rng(92)
    n = 30000
    pos = torch.tensor(learned.mixture_positions(n, seed=92), device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (n, 1)), device="cuda")
    t = fg.build_tree(pos, S, n, 64, 10, 0.5)
    model = learned.OrderModel(seed=4)
    model.attach(t, 0.05)
    ref = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.set_graph(True)
    F = torch.empty((n, 4), dtype=torch.float64, device="cuda")
    for _ in range(3):
        F.zero_()
        t.compute_field_fmm(F, precision="mixed")
        assert np.array_equal(F.cpu().numpy(), ref)
    # detaching the model re-records the fixed-order pass
    t.set_order_model(None)
    fixed = fg.build_tree(pos, S, n, 64, 10, 0.5).compute_field_fmm(precision="mixed").cpu().numpy()
    for _ in range(2):
        t.compute_field_fmm(F, precision="mixed")
        assert np.array_equal(F.cpu().numpy(), fixed)


# ---------------------------------------------------------------------------
# what the trained model gains
# ---------------------------------------------------------------------------
def test_trained_model_gain(fg):
    """The committed p_max = 12 model on an unseen clustered system: the field
    error stays at the 1e-6 target while the M2L does a fraction of the fixed
    p = 12 work, and less than the cheapest fixed order that reaches the same
    error."""
    from fmmgen_gb300 import learned

    if not os.path.exists(learned.MODEL_PATH):
        pytest.skip("no trained order model committed")
    model = learned.OrderModel.load()
    n = 400_000
    rng = np.random.default_rng(4242)
    pos = torch.tensor(learned.mixture_positions(n, seed=4242), device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (n, 1)), device="cuda")
    targets = np.sort(rng.choice(n, 4000, replace=False))
    Fd = fg.direct(pos, S, targets=targets, potential=False, field=True).cpu().numpy()

    def err(t, prec):
        return rel(t.compute_field_fmm(potential=False, field=True, precision=prec).cpu().numpy()[targets], Fd)

    t = fg.build_tree(pos, S, n, 128, 12, 0.5)
    e12 = err(t, "mixed")
    model.attach(t)
    eL = err(t, "mixed")
    wL = learned.m2l_terms(t.m2l_orders())
    w12 = t.nm2l * learned.pair_terms(12)
    fixed = {}
    for q in range(6, 12):
        fixed[q] = err(fg.build_tree(pos, S, n, 128, q, 0.5), "mixed")
    qstar = min([q for q in fixed if fixed[q] <= eL] + [12])
    wq = t.nm2l * learned.pair_terms(qstar)
    print(f"fixed p=12 error {e12:.3e}; learned error {eL:.3e}; fixed errors "
          + ", ".join(f"p={q}: {e:.2e}" for q, e in fixed.items())
          + f"; M2L multiply-adds learned {wL:.3e}, fixed p=12 {w12:.3e}, fixed p={qstar} {wq:.3e}")
    assert eL <= 1e-6
    assert wL < w12 / 3
    assert wL < wq
