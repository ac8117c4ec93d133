"""Batched device operators (and the scalar twins of the generated ABI) against
fmmgen's generated operators: FP64, 1e-12 relative on identical inputs."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
TOL = 1e-12  # max-norm relative, per output vector


def relerr(a, b):
    return np.max(np.abs(a - b), axis=-1) / np.maximum(np.max(np.abs(b), axis=-1), 1e-300)


def cu(a):
    return torch.tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("so", [0, 1])
def test_batched_ops_vs_generated(fg, so):
    ops = fg.operators
    g = np.load(os.path.join(GOLDEN, f"ops_so{so}.npz"))
    for p in range(int(g["pmin"]), int(g["pmax"]) + 1):
        d, q, Min, Lin = g[f"p{p}_d"], g[f"p{p}_q"], g[f"p{p}_M"], g[f"p{p}_L"]
        K = len(d)
        ms, ls = ops.msize(p, so), ops.lsize(p, so)
        M = torch.zeros(K, ms, dtype=torch.float64, device="cuda")
        ops.P2M_batch(cu(d), cu(q), M, p, so)
        assert relerr(M.cpu().numpy(), g[f"p{p}_P2M"]).max() < TOL
        Ms = torch.zeros(K, ms, dtype=torch.float64, device="cuda")
        ops.M2M_batch(cu(d), cu(Min), Ms, p, so)
        assert relerr(Ms.cpu().numpy(), g[f"p{p}_M2M"]).max() < TOL
        L = torch.zeros(K, ls, dtype=torch.float64, device="cuda")
        ops.M2L_batch(cu(d), cu(Min), L, p, so)
        assert relerr(L.cpu().numpy(), g[f"p{p}_M2L"]).max() < TOL, p
        Ls = torch.zeros(K, ls, dtype=torch.float64, device="cuda")
        ops.L2L_batch(cu(d), cu(Lin), Ls, p, so)
        assert relerr(Ls.cpu().numpy(), g[f"p{p}_L2L"]).max() < TOL
        F = torch.zeros(K, 4, dtype=torch.float64, device="cuda")
        ops.L2P_batch(cu(d), cu(Lin), F, p, so)
        assert relerr(F.cpu().numpy(), g[f"p{p}_L2P"]).max() < TOL
    F = torch.zeros(len(g["p2p_d"]), 4, dtype=torch.float64, device="cuda")
    ops.P2P_batch(cu(g["p2p_d"]), cu(g["p2p_S"]), F, so)
    assert relerr(F.cpu().numpy(), g["p2p_F"]).max() < 1e-14


@pytest.mark.parametrize("p,so", [(10, 0), (12, 0), (8, 1), (12, 1)])
def test_batched_ops_high_order_vs_oracle(fg, oracle_lib, p, so):
    """Orders beyond the generated fixtures, against the CPU restatement."""
    ops, O = fg.operators, oracle_lib
    rng = np.random.default_rng(p + 100 * so)
    K = 64
    d = rng.uniform(-1, 1, (K, 3))
    d *= rng.uniform(2.0, 4.0, (K, 1)) / np.linalg.norm(d, axis=1, keepdims=True)
    ms, ls = O.msize(p, so), O.lsize(p, so)
    Min, Lin = rng.standard_normal((K, ms)), rng.standard_normal((K, ls))
    ref_M2L = np.zeros((K, ls))
    ref_M2M = np.zeros((K, ms))
    ref_L2L = np.zeros((K, ls))
    for i in range(K):
        O.M2L(*d[i], Min[i].copy(), ref_M2L[i], p, so)
        O.M2M(*d[i], Min[i].copy(), ref_M2M[i], p, so)
        O.L2L(*d[i], Lin[i].copy(), ref_L2L[i], p, so)
    L = torch.zeros(K, ls, dtype=torch.float64, device="cuda")
    ops.M2L_batch(cu(d), cu(Min), L, p, so)
    # per-degree scaled error: high-order derivative blocks shrink like |d|^-(|k|+1)
    assert relerr(L.cpu().numpy(), ref_M2L).max() < 1e-11
    Ms = torch.zeros(K, ms, dtype=torch.float64, device="cuda")
    ops.M2M_batch(cu(d), cu(Min), Ms, p, so)
    assert relerr(Ms.cpu().numpy(), ref_M2M).max() < TOL
    Ls = torch.zeros(K, ls, dtype=torch.float64, device="cuda")
    ops.L2L_batch(cu(d), cu(Lin), Ls, p, so)
    assert relerr(Ls.cpu().numpy(), ref_L2L).max() < TOL


def test_accumulate_semantics(fg):
    """Outputs are added to, never overwritten (the generated `+=`)."""
    ops = fg.operators
    d = cu([[1.5, -0.5, 2.0]])
    M = cu(np.arange(35, dtype=np.float64)[None, :] / 7.0)
    L0 = np.linspace(-1, 1, 35)[None, :]
    L = cu(L0)
    ops.M2L_batch(d, M, L, 4, 0)
    L1 = cu(np.zeros((1, 35)))
    ops.M2L_batch(d, M, L1, 4, 0)
    assert np.allclose(L.cpu().numpy(), L0 + L1.cpu().numpy(), rtol=1e-15, atol=1e-15)


def test_scalar_twins_known_answers(fg):
    """tests/test_multipoles.py of the reference, through the scalar M2M twin."""
    m = fg.operators.module(5, source_order=0)
    for order in range(1, m.FMMGEN_MAXORDER):
        d, q = 1.0, 5.0
        M = np.zeros(fg.operators.nterms(order))
        for x, s in ((np.array([d, 0, 0]), q), (np.array([-d, 0, 0]), -q)):
            S = np.zeros(fg.operators.nterms(order)); S[0] = s
            m.M2M(*(-x), S, M, order)
        assert M[0] == 0.0 and M[1] == -2 * q * d and M[2] == 0.0 and M[3] == 0.0
    for order in range(2, m.FMMGEN_MAXORDER):
        d, q = 2.0, 5.0
        M = np.zeros(fg.operators.nterms(order))
        for x, s in ((np.array([-d, 0, 0]), -q), (np.array([d, 0, 0]), -q), (np.zeros(3), 2 * q)):
            S = np.zeros(fg.operators.nterms(order)); S[0] = s
            m.M2M(*(-x), S, M, order)
        assert M[:4].tolist() == [0.0, 0.0, 0.0, 0.0] and M[4] == -2 * d * q
    # out-of-range order is a silent no-op, as in the generated switch
    M = np.zeros(35)
    m.M2M(1.0, 0.0, 0.0, np.ones(35), M, 7)
    assert not M.any()


def test_scalar_twin_m2l_l2p_chain(fg, oracle_lib):
    """M2M -> M2L -> L2L -> L2P on the scalar twins vs the checker."""
    m = fg.operators.module(9, source_order=0)
    O = oracle_lib
    p = 8
    M = np.zeros(165); Mo = np.zeros(165)
    S = np.zeros(165); S[0] = 0.7
    m.M2M(0.1, -0.2, 0.05, S, M, p); O.M2M(0.1, -0.2, 0.05, S, Mo, p)
    L = np.zeros(165); Lo = np.zeros(165)
    m.M2L(3.0, 1.0, -2.0, M, L, p); O.M2L(3.0, 1.0, -2.0, Mo, Lo, p)
    Ls = np.zeros(165); Lso = np.zeros(165)
    m.L2L(0.2, 0.1, -0.1, L, Ls, p); O.L2L(0.2, 0.1, -0.1, Lo, Lso, p)
    F = np.zeros(4); Fo = np.zeros(4)
    m.L2P(0.05, 0.02, 0.01, Ls, F, p); O.L2P(0.05, 0.02, 0.01, Lso, Fo, p)
    assert np.max(np.abs(F - Fo)) < 1e-12 * np.max(np.abs(Fo))
