"""The precision="float" operator variant (fmmgen/writer.py:105): the FP32
batched operators and scalar twins against the reference's own float operators
(tests/golden/ops_f32_so*.npz, generated with precision="float") and the FP64
generated operators (ops_so*.npz).  Both FP32 codes get the same
float32-rounded inputs; each is scored by its distance from the FP64 answer,
and ours may be at most a small factor above the reference's."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
OPS = ("P2M", "M2M", "M2L", "L2L", "L2P")
FACTOR, FLOOR = 4.0, 1e-6   # ours <= FACTOR x the reference float error + FLOOR


def relerr(a, b):
    return (np.max(np.abs(a - b), axis=-1) / np.max(np.abs(b), axis=-1)).max()


def cu32(a):
    return torch.tensor(np.ascontiguousarray(a, dtype=np.float32), device="cuda")


@pytest.mark.parametrize("so", [0, 1, 2])
def test_batched_f32_vs_reference_float(fg, so):
    ops = fg.operators
    g = np.load(os.path.join(GOLDEN, f"ops_so{so}.npz"))
    f = np.load(os.path.join(GOLDEN, f"ops_f32_so{so}.npz"))
    for p in range(int(g["pmin"]), int(g["pmax"]) + 1):
        d, q, Min, Lin = (cu32(g[f"p{p}_{k}"]) for k in "dqML")
        K, ms, ls = d.shape[0], ops.msize(p, so), ops.lsize(p, so)
        out = {k: torch.zeros(K, w, dtype=torch.float32, device="cuda")
               for k, w in (("P2M", ms), ("M2M", ms), ("M2L", ls), ("L2L", ls), ("L2P", 4))}
        ops.P2M_batch(d, q, out["P2M"], p, so)
        ops.M2M_batch(d, Min, out["M2M"], p, so)
        ops.M2L_batch(d, Min, out["M2L"], p, so)
        ops.L2L_batch(d, Lin, out["L2L"], p, so)
        ops.L2P_batch(d, Lin, out["L2P"], p, so)
        for k in OPS:
            truth = g[f"p{p}_{k}"]
            ours = relerr(out[k].cpu().numpy().astype(np.float64), truth)
            ref = relerr(f[f"p{p}_{k}"].astype(np.float64), truth)
            assert ours <= FACTOR * ref + FLOOR, (so, p, k, ours, ref)
    F = torch.zeros(len(g["p2p_d"]), 4, dtype=torch.float32, device="cuda")
    ops.P2P_batch(cu32(g["p2p_d"]), cu32(g["p2p_S"]), F, so)
    Fn = F.cpu().numpy().astype(np.float64)
    ref_phi = np.max(np.abs(f["p2p_phi"] - g["p2p_F"][:, 0])) / np.max(np.abs(g["p2p_F"][:, 0]))
    assert np.max(np.abs(Fn[:, 0] - g["p2p_F"][:, 0])) / np.max(np.abs(g["p2p_F"][:, 0])) <= FACTOR * ref_phi + FLOOR
    assert relerr(Fn[:, 1:], g["p2p_F"][:, 1:]) < 1e-6


@pytest.mark.parametrize("so", [0, 1, 2])
def test_f32_m2p_potential(fg, so):
    """M2P in FP32 against the FP64 generated potential."""
    name = "m2p_potential_so2.npz" if so == 2 else "m2p_potential.npz"
    m = np.load(os.path.join(GOLDEN, name))
    orders = [int(k.split("_")[1][1:]) for k in m.files if k.startswith(f"so{so}_") and k.endswith("_phi")]
    assert orders
    for p in orders:
        d, Mv, phi = m[f"so{so}_p{p}_d"], m[f"so{so}_p{p}_M"], m[f"so{so}_p{p}_phi"]
        F = torch.zeros(len(d), 1, dtype=torch.float32, device="cuda")
        fg.operators.M2P_batch(cu32(d), cu32(Mv), F, p, so, potential=True, field=False)
        err = np.max(np.abs(F.cpu().numpy()[:, 0].astype(np.float64) - phi)) / np.max(np.abs(phi))
        assert err < 1e-4, (so, p, err)


def test_f32_matches_f64_kernels_in_bulk(fg):
    """Many random applications at the highest order: the FP32 kernels against
    the FP64 kernels of the same operators (bounded by float rounding)."""
    ops = fg.operators
    rng = np.random.default_rng(11)
    K, p, so = 4096, 12, 0
    d = rng.uniform(-1, 1, (K, 3))
    d *= rng.uniform(1.5, 3.0, (K, 1)) / np.linalg.norm(d, axis=1, keepdims=True)
    d = d.astype(np.float32).astype(np.float64)
    M = rng.standard_normal((K, ops.msize(p, so))).astype(np.float32).astype(np.float64)
    L64 = torch.zeros(K, ops.lsize(p, so), dtype=torch.float64, device="cuda")
    ops.M2L_batch(torch.tensor(d, device="cuda"), torch.tensor(M, device="cuda"), L64, p, so)
    L32 = torch.zeros(K, ops.lsize(p, so), dtype=torch.float32, device="cuda")
    ops.M2L_batch(cu32(d), cu32(M), L32, p, so)
    a, b = L32.double().cpu().numpy(), L64.cpu().numpy()
    assert relerr(a, b) < 1e-3


def test_dtype_mismatch_rejected(fg):
    ops = fg.operators
    d = torch.zeros(2, 3, dtype=torch.float32, device="cuda")
    q = torch.zeros(2, dtype=torch.float64, device="cuda")
    M = torch.zeros(2, ops.msize(4, 0), dtype=torch.float32, device="cuda")
    with pytest.raises(TypeError):
        ops.P2M_batch(d, q, M, 4, 0)


@pytest.mark.parametrize("so", [0, 1, 2])
def test_float_module_scalar_twins(fg, so):
    """module(..., precision="float"): float[:] buffers, the generated float
    names and order rules; values against the reference's float operators."""
    g = np.load(os.path.join(GOLDEN, f"ops_so{so}.npz"))
    f = np.load(os.path.join(GOLDEN, f"ops_f32_so{so}.npz"))
    pmax = int(g["pmax"])
    m = fg.operators.module(pmax + 1, source_order=so, precision="float")
    assert m.precision == "float"
    for p in (int(g["pmin"]), pmax):
        d, q, Min, Lin = (g[f"p{p}_{k}"].astype(np.float32) for k in "dqML")
        for i in range(2):
            x, y, z = (float(v) for v in d[i])
            outs = {}
            a = np.zeros(Min.shape[1], np.float32); m.P2M(x, y, z, float(q[i]), a, p); outs["P2M"] = a
            a = np.zeros(Min.shape[1], np.float32); m.M2M(x, y, z, Min[i].copy(), a, p); outs["M2M"] = a
            a = np.zeros(Lin.shape[1], np.float32); m.M2L(x, y, z, Min[i].copy(), a, p); outs["M2L"] = a
            a = np.zeros(Lin.shape[1], np.float32); m.L2L(x, y, z, Lin[i].copy(), a, p); outs["L2L"] = a
            a = np.zeros(4, np.float32); getattr(m, f"L2P{p}")(x, y, z, Lin[i].copy(), a); outs["L2P"] = a
            for k, v in outs.items():
                truth = g[f"p{p}_{k}"][i]
                ours = relerr(v.astype(np.float64), truth)
                ref = relerr(f[f"p{p}_{k}"][i].astype(np.float64), truth)
                assert ours <= FACTOR * ref + FLOOR, (so, p, k, ours, ref)
    with pytest.raises(TypeError):
        m.M2M(0.1, 0.2, 0.3, np.zeros(Min.shape[1]), np.zeros(Min.shape[1]), pmax)
