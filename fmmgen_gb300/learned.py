"""Learned per-pair M2L orders (no counterpart in the reference, whose FMM
applies one expansion order to every M2L pair: example/calculate.cpp:190-206).

A small MLP (16 -> 64 -> 64 -> 11, ReLU, FP32) reads features of an M2L pair
B -> A -- the level difference, the separation in target half-widths, the
per-degree norms of B's multipole folded into the pair's estimated far field,
and that estimate against the pair's share of the error budget -- and predicts
the lowest order q in 2..12 whose truncation keeps the pair's field error in
the target cell within its share.  The budget is global: a relative L2 field
error eps over the system, its square split equally over the system's M2L
pairs, scaled by the near-field (P2P) RMS of the same pass.  The tree then applies each
pair at its own order (the terms |n| + |m| <= q of the order-p translation).
The fixed-order FMM stays the fallback (detach the model) and the judge of the
error.  Features, labels, inference and the whole training step (forward,
backward, weight gradients, Adam) are hand-written kernels in
libfmmgen_gb300.so (csrc/learn.cu); torch only holds the buffers and draws the
minibatch indices.

    model = OrderModel.load()                    # the committed p_max = 12 model
    tree = build_tree(pos, S, N, 128, 12, 0.5)
    model.attach(tree)                           # tree.set_order_model(params, delta, eps)
    F = tree.compute_field_fmm(precision="mixed")

Training data come from the plain fixed-order FMM (`training_pairs`): an FP64
pass at p_max, the features of its pairs, and labels from its own multipoles
(the exact truncation error of each pair at every order, bounded over the
target cell).
`python -m fmmgen_gb300.learned --out model.npz` trains a model from scratch.
"""
import argparse
import ctypes as C
import math
import os
import time

import numpy as np
import torch

from ._lib import check, lib
from .tree import _stream_ptr

NFEAT, NCLS, QMIN = 16, 11, 2
MODEL_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "order_model_p12_so0.npz")


def nparam():
    return int(lib().fmmgen_order_model_nparam())


def _ptr(t):
    return C.c_void_p(t.data_ptr())


# ---------------------------------------------------------------------------
# features, labels, work
# ---------------------------------------------------------------------------
def order_features(tree, eps=1e-6, stream=None):
    """Features [nm2l][16] (float32, device) of every M2L pair, export_lists
    order, from the multipoles and near field of the tree's last evaluation,
    for the relative field error target eps."""
    feat = torch.empty((max(tree.nm2l, 1), NFEAT), dtype=torch.float32, device="cuda")
    check(lib().fmmgen_tree_order_features(tree._h, float(eps), _ptr(feat), _stream_ptr(stream)))
    return feat[: tree.nm2l]


def order_labels(tree, eps=1e-6, errq=False, stream=None):
    """Labels (uint8, device; order - 2) of every M2L pair after an FP64
    evaluation; with errq also the bound at orders 2..12 over the pair's
    budget ([nm2l][11] float32)."""
    n = max(tree.nm2l, 1)
    lab = torch.empty(n, dtype=torch.uint8, device="cuda")
    eq = torch.empty((n, NCLS), dtype=torch.float32, device="cuda") if errq else None
    check(lib().fmmgen_tree_order_labels(tree._h, float(eps), _ptr(lab), _ptr(eq) if eq is not None else None,
                                         _stream_ptr(stream)))
    if errq:
        return lab[: tree.nm2l], eq[: tree.nm2l]
    return lab[: tree.nm2l]


def _nterms(p):
    return (p + 1) * (p + 2) * (p + 3) // 6 if p >= 0 else 0


def pair_terms(q, so=0):
    """Multiply-adds of one M2L pair at order q: the (n, m) with |m| >= so, |n| + |m| <= q."""
    return sum((d + 1) * (d + 2) // 2 * _nterms(q - d) for d in range(so, q + 1))


def m2l_terms(orders, so=0):
    """Multiply-adds of an M2L pass whose pair k runs at order orders[k]."""
    o = np.asarray(orders.cpu() if isinstance(orders, torch.Tensor) else orders, dtype=np.int64)
    h = np.bincount(o, minlength=13)
    return int(sum(int(h[q]) * pair_terms(q, so) for q in range(len(h)) if h[q]))


# ---------------------------------------------------------------------------
# kernels
# ---------------------------------------------------------------------------
def predict(params, feat, delta=0.0, qmax=12, stream=None):
    """Orders (uint8, device) of feature rows: the lowest q whose cumulative
    predicted probability reaches 1 - delta, clamped to [2, qmax]."""
    n = feat.shape[0]
    out = torch.empty(max(n, 1), dtype=torch.uint8, device="cuda")
    check(lib().fmmgen_mlp_predict(_ptr(params), _ptr(feat), n, float(delta), int(qmax), _ptr(out),
                                   _stream_ptr(stream)))
    return out[:n]


def train_step(params, X, y, grad, loss, work=None, stream=None):
    """Gradient (into grad) and mean cross-entropy (added to the device scalar
    loss) of the model on the rows X with labels y."""
    n = X.shape[0]
    if work is None or work.numel() < lib().fmmgen_mlp_train_work(n):
        work = torch.empty(int(lib().fmmgen_mlp_train_work(n)), dtype=torch.float32, device="cuda")
    check(lib().fmmgen_mlp_train_step(_ptr(params), _ptr(X), _ptr(y), n, _ptr(grad), _ptr(loss), _ptr(work),
                                      _stream_ptr(stream)))
    return work


def adam_step(params, grad, m, v, step, lr, stream=None):
    check(lib().fmmgen_mlp_adam(_ptr(params), _ptr(grad), _ptr(m), _ptr(v), int(step), float(lr),
                                _stream_ptr(stream)))


# ---------------------------------------------------------------------------
# the model
# ---------------------------------------------------------------------------
_LAYERS = [(64, 16), (64, 64), (11, 64)]


def init_params(seed=0):
    """He-initialised parameters (host float32, the device layout)."""
    rng = np.random.default_rng(seed)
    parts = []
    for fo, fi in _LAYERS:
        parts.append(rng.standard_normal((fo, fi)) * math.sqrt(2.0 / fi))
        parts.append(np.zeros(fo))
    return np.concatenate([p.ravel() for p in parts]).astype(np.float32)


def fold_normalisation(params, mean, std):
    """Parameters acting on raw features x of a model trained on (x - mean) / std."""
    p = np.asarray(params, dtype=np.float64).copy()
    W1 = p[: 64 * 16].reshape(64, 16)
    b1 = p[64 * 16: 64 * 16 + 64]
    W1n = W1 / std[None, :]
    p[: 64 * 16] = W1n.ravel()
    p[64 * 16: 64 * 16 + 64] = b1 - W1n @ mean
    return p.astype(np.float32)


class OrderModel:
    """Order-model parameters on the device, the decoding threshold delta and
    the error target eps the model was trained for."""

    def __init__(self, params=None, delta=0.0, seed=0, meta=None, eps=1e-6):
        host = init_params(seed) if params is None else np.asarray(params, dtype=np.float32).ravel()
        if host.size != nparam():
            raise ValueError(f"an order model has {nparam()} parameters, got {host.size}")
        self.params = torch.tensor(host, device="cuda")
        self.delta = float(delta)
        self.meta = dict(meta or {})
        self.eps = float(self.meta.get("eps", eps))

    @classmethod
    def load(cls, path=MODEL_PATH):
        z = np.load(path, allow_pickle=False)
        meta = {k: z[k].item() if z[k].ndim == 0 else z[k] for k in z.files if k not in ("params", "delta")}
        return cls(z["params"], float(z["delta"]), meta=meta)

    def save(self, path, **meta):
        m = dict(self.meta)
        m.update(meta)
        np.savez(path, params=self.params.cpu().numpy(), delta=np.float64(self.delta),
                 **{k: np.asarray(v) for k, v in m.items()})

    def predict(self, feat, delta=None, qmax=12, stream=None):
        return predict(self.params, feat, self.delta if delta is None else delta, qmax, stream)

    def attach(self, tree, delta=None):
        tree.set_order_model(self.params, self.delta if delta is None else delta, self.eps)
        return tree

    def fit(self, X, y, steps=3000, batch=65536, lr=3e-3, lr_final=1e-4, seed=0, log_every=0):
        """Train from the current parameters on rows X (float32 [n][16], device)
        with labels y (uint8 [n], device): Adam on minibatch cross-entropy with
        the features normalised by their mean and spread (folded back into the
        first layer at the end), learning rate decayed geometrically from lr to
        lr_final.  Returns the mean loss of each logged interval."""
        n = X.shape[0]
        mean = X.double().mean(0)
        std = X.double().std(0).clamp_min(1e-3)
        Xn = ((X.double() - mean) / std).float().contiguous()
        mean_h, std_h = mean.cpu().numpy(), std.cpu().numpy()
        P = self.params
        grad = torch.zeros_like(P)
        m = torch.zeros_like(P)
        v = torch.zeros_like(P)
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        work = torch.empty(int(lib().fmmgen_mlp_train_work(batch)), dtype=torch.float32, device="cuda")
        g = torch.Generator(device="cuda")
        g.manual_seed(seed)
        hist, last = [], 0
        log_every = log_every or max(1, steps // 20)
        for t in range(1, steps + 1):
            idx = torch.randint(0, n, (batch,), device="cuda", generator=g)
            xb = Xn.index_select(0, idx).contiguous()
            yb = y.index_select(0, idx).contiguous()
            train_step(P, xb, yb, grad, loss, work)  # adds this minibatch's mean loss
            lr_t = lr * (lr_final / lr) ** ((t - 1) / max(1, steps - 1))
            adam_step(P, grad, m, v, t, lr_t)
            if t % log_every == 0 or t == steps:
                hist.append(float(loss.item()) / (t - last))
                loss.zero_()
                last = t
        self.params = torch.tensor(fold_normalisation(P.cpu().numpy(), mean_h, std_h), device="cuda")
        return hist


# ---------------------------------------------------------------------------
# training data
# ---------------------------------------------------------------------------
def mixture_positions(n, nclusters=64, sigma=0.01, seed=0):
    """n positions: the first half uniform in the unit cube, the rest in
    nclusters isotropic Gaussian clusters (centres uniform in the cube)."""
    rng = np.random.default_rng(seed)
    nu = n // 2
    centres = rng.uniform(0, 1, (nclusters, 3))
    which = rng.integers(0, nclusters, n - nu)
    return np.concatenate([rng.uniform(0, 1, (nu, 3)), centres[which] + sigma * rng.standard_normal((n - nu, 3))])


def training_pairs(tree, eps):
    """Features and labels of every M2L pair of a built tree (with its sources
    set) from one FP64 pass at the tree's order."""
    tree.compute_field_fmm(potential=True, field=True, precision="fp64")
    return order_features(tree, eps), order_labels(tree, eps)


def _rel_err(F, R):
    return float(np.linalg.norm(F - R) / np.linalg.norm(R))


def calibrate_delta(model, tree, targets, Fdirect, target_err,
                    deltas=(1e-3, 1e-2, 3e-2, 0.1, 0.2, 0.3, 0.5, 0.6, 0.7, 0.8, 0.9), precision="mixed"):
    """Largest delta (cheapest orders) whose field error on `targets` against
    Fdirect ([len(targets)][3], the direct sum) stays within target_err;
    returns (delta, {delta: (error, M2L multiply-adds)})."""
    table = {}
    best = min(deltas)
    for d in sorted(deltas):
        model.attach(tree, d)
        F = tree.compute_field_fmm(potential=False, field=True, precision=precision).cpu().numpy()[targets]
        e = _rel_err(F, Fdirect)
        table[d] = (e, m2l_terms(tree.m2l_orders(), tree.source_order))
        if e <= target_err:
            best = d
    tree.set_order_model(None)
    return best, table


def main(argv=None):
    from .tree import build_tree, direct

    ap = argparse.ArgumentParser(description="train the per-pair M2L order model")
    ap.add_argument("--out", default=MODEL_PATH)
    ap.add_argument("--pairs", type=float, default=10e6, help="training pairs to collect")
    ap.add_argument("--n", type=int, default=1_000_000, help="particles per training system")
    ap.add_argument("--order", type=int, default=12)
    ap.add_argument("--eps", type=float, default=5e-6, help="error target of the labels and features")
    ap.add_argument("--target-err", type=float, default=0.8e-6,
                    help="field error the decoding threshold is calibrated to (a margin below 1e-6)")
    ap.add_argument("--steps", type=int, default=4000)
    ap.add_argument("--batch", type=int, default=65536)
    ap.add_argument("--seed", type=int, default=1000)
    a = ap.parse_args(argv)
    t0 = time.time()
    Xs, ys, seed, got = [], [], a.seed, 0
    while got < a.pairs:
        rng = np.random.default_rng(seed)
        pos = mixture_positions(a.n, nclusters=int(rng.integers(8, 129)), sigma=float(rng.uniform(0.005, 0.03)),
                                seed=seed)
        S = rng.uniform(-1, 1, (a.n, 1))
        tree = build_tree(pos, S, a.n, 128, a.order, 0.5)
        X, y = training_pairs(tree, a.eps)
        Xs.append(X.clone())
        ys.append(y.clone())
        got += X.shape[0]
        print(f"system seed {seed}: {X.shape[0]} pairs (total {got})", flush=True)
        seed += 1
        del tree
    X = torch.cat(Xs)
    y = torch.cat(ys)
    hist = np.bincount(y.cpu().numpy(), minlength=NCLS)
    print("labels (orders 2..12):", hist.tolist(), flush=True)
    model = OrderModel(seed=a.seed, eps=a.eps)
    losses = model.fit(X, y, steps=a.steps, batch=a.batch)
    print("loss:", " ".join(f"{v:.4f}" for v in losses), flush=True)
    # calibrate delta on a held-out system
    n = a.n // 2
    rng = np.random.default_rng(seed + 7)
    pos = mixture_positions(n, seed=seed + 7)
    S = rng.uniform(-1, 1, (n, 1))
    tree = build_tree(pos, S, n, 128, a.order, 0.5)
    targets = np.sort(rng.choice(n, 5000, replace=False))
    Fd = direct(tree.pos, tree.S, targets=targets, potential=False, field=True).cpu().numpy()
    delta, table = calibrate_delta(model, tree, targets, Fd, a.target_err)
    for d, (e, w) in table.items():
        print(f"delta {d:g}: field error {e:.3e}, M2L multiply-adds {w:.4g}", flush=True)
    # the labels themselves as orders, and the fixed orders, on the same system
    _, Xv = None, training_pairs(tree, a.eps)
    tree.set_m2l_orders(Xv[1].to(torch.uint8) + QMIN)
    F = tree.compute_field_fmm(potential=False, field=True, precision="mixed").cpu().numpy()[targets]
    print(f"label orders: field error {_rel_err(F, Fd):.3e}, M2L multiply-adds "
          f"{m2l_terms(Xv[1].cpu().numpy().astype(np.int64) + QMIN):.4g}", flush=True)
    tree.set_m2l_orders(None)
    for q in range(6, a.order + 1):
        tq = build_tree(tree.pos, tree.S, n, 128, q, 0.5)
        F = tq.compute_field_fmm(potential=False, field=True, precision="mixed").cpu().numpy()[targets]
        print(f"fixed p={q}: field error {_rel_err(F, Fd):.3e}, M2L multiply-adds {tq.nm2l * pair_terms(q):.4g}",
              flush=True)
    model.delta = delta
    model.save(a.out, order=a.order, eps=a.eps, target_err=a.target_err, pairs=int(X.shape[0]),
               label_hist=hist, loss=np.asarray(losses), train_seconds=time.time() - t0)
    print(f"saved {a.out} (delta {delta:g}) in {time.time() - t0:.1f} s", flush=True)


if __name__ == "__main__":
    main()
