"""Quadrupole sources (source_order 2): the batched operators against fmmgen's
generated operators, and the whole evaluation pass (FP64 and mixed) against the
reference's compute_field_fmm on a quadrupole Plummer tree (tests/golden), the
CPU restatement's direct sum and Barnes-Hut pass."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
TOL_OPS = 1e-12
TOL_FP64 = 1e-10
TOL_MIXED = 2e-6


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def relerr(a, b):
    return np.max(np.abs(a - b), axis=-1) / np.maximum(np.max(np.abs(b), axis=-1), 1e-300)


def cu(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


def test_batched_ops_vs_generated(fg):
    ops = fg.operators
    so = 2
    g = np.load(os.path.join(GOLDEN, "ops_so2.npz"))
    for p in range(int(g["pmin"]), int(g["pmax"]) + 1):
        d, q, Min, Lin = g[f"p{p}_d"], g[f"p{p}_q"], g[f"p{p}_M"], g[f"p{p}_L"]
        K = len(d)
        ms, ls = ops.msize(p, so), ops.lsize(p, so)
        M = torch.zeros(K, ms, dtype=torch.float64, device="cuda")
        ops.P2M_batch(cu(d), cu(q), M, p, so)
        assert relerr(M.cpu().numpy(), g[f"p{p}_P2M"]).max() < TOL_OPS
        Ms = torch.zeros(K, ms, dtype=torch.float64, device="cuda")
        ops.M2M_batch(cu(d), cu(Min), Ms, p, so)
        assert relerr(Ms.cpu().numpy(), g[f"p{p}_M2M"]).max() < TOL_OPS
        L = torch.zeros(K, ls, dtype=torch.float64, device="cuda")
        ops.M2L_batch(cu(d), cu(Min), L, p, so)
        assert relerr(L.cpu().numpy(), g[f"p{p}_M2L"]).max() < TOL_OPS, p
        Ls = torch.zeros(K, ls, dtype=torch.float64, device="cuda")
        ops.L2L_batch(cu(d), cu(Lin), Ls, p, so)
        assert relerr(Ls.cpu().numpy(), g[f"p{p}_L2L"]).max() < TOL_OPS
        F = torch.zeros(K, 4, dtype=torch.float64, device="cuda")
        ops.L2P_batch(cu(d), cu(Lin), F, p, so)
        assert relerr(F.cpu().numpy(), g[f"p{p}_L2P"]).max() < TOL_OPS
    F = torch.zeros(len(g["p2p_d"]), 4, dtype=torch.float64, device="cuda")
    ops.P2P_batch(cu(g["p2p_d"]), cu(g["p2p_S"]), F, so)
    assert relerr(F.cpu().numpy(), g["p2p_F"]).max() < 1e-13
    # the generated potential, through M2P at every order
    m = np.load(os.path.join(GOLDEN, "m2p_potential_so2.npz"))
    for p in range(3, 6):
        d, Mv, phi = m[f"so2_p{p}_d"], m[f"so2_p{p}_M"], m[f"so2_p{p}_phi"]
        F = torch.zeros(len(d), 1, dtype=torch.float64, device="cuda")
        ops.M2P_batch(cu(d), cu(Mv), F, p, so, potential=True, field=False)
        assert np.max(np.abs(F.cpu().numpy()[:, 0] - phi)) <= 1e-12 * np.max(np.abs(phi))


def load_tree(fg, precision="fp64"):
    g = np.load(os.path.join(GOLDEN, "tree_quadrupole_plummer.npz"))
    assert int(g["source_order"]) == 2 and g["S"].shape[1] == 6
    pos, S = cu(g["pos"]), cu(g["S"])
    t = fg.build_tree(pos, S, int(g["N"]), int(g["ncrit"]), int(g["order"]), float(g["theta"]), source_order=2)
    return g, t, t.compute_field_fmm(precision=precision).cpu().numpy()


def test_fp64_fmm_vs_reference(fg):
    g, _, F = load_tree(fg, "fp64")
    assert rel(F, g["F"]) < TOL_FP64


@pytest.mark.parametrize("precision", ["mixed", "mixed_simt"])
def test_mixed_fmm_vs_reference(fg, precision):
    g, _, F = load_tree(fg, precision)
    assert rel(F[:, 1:], g["F"][:, 1:]) < TOL_MIXED
    assert rel(F[:, 0], g["F"][:, 0]) < TOL_MIXED


def test_direct_and_bh_vs_checker(fg, oracle_lib):
    g, t, _ = load_tree(fg)
    idx = np.arange(0, int(g["N"]), 11)
    Fd = t.compute_field_exact(targets=idx).cpu().numpy()
    Fo = oracle_lib.direct(g["pos"], g["S"], idx, source_order=2)
    assert rel(Fd, Fo) < 1e-12
    Fb = t.compute_field_bh().cpu().numpy()
    ot = oracle_lib.OracleTree(g["pos"], g["S"], int(g["ncrit"]), int(g["order"]), float(g["theta"]), 2)
    Fbo = ot.evaluate_bh()
    assert rel(Fb, Fbo) < 1e-10


def test_fused_equals_two_calls(fg):
    g = np.load(os.path.join(GOLDEN, "tree_quadrupole_plummer.npz"))
    pos, S = cu(g["pos"]), cu(g["S"])
    n, ncrit, p, th = int(g["N"]), int(g["ncrit"]), int(g["order"]), float(g["theta"])
    a = fg.build_tree(pos, S, n, ncrit, p, th, source_order=2)
    b = fg.build_tree(pos, S, n, ncrit, p, th, source_order=2)
    for precision in ("fp64", "mixed"):
        Fa = a.compute_field_fmm(precision=precision).cpu().numpy()
        Fb = b.rebuild_compute(pos, precision=precision).cpu().numpy()
        assert np.array_equal(Fa, Fb)
