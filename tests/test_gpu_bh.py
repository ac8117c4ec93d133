"""Barnes-Hut on the GPU (Tree::compute_field_bh): potentials against the
reference's own (tests/golden/bh_*.npz), fields against the oracle's walk with
the physical M2P field, the output switches, and forests against separate
trees."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
CASES = ["uniform10k", "clustered", "dipole_plummer"]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("name", CASES)
def test_bh_matches_reference_and_oracle(fg, oracle_lib, name):
    g = np.load(os.path.join(GOLDEN, f"bh_{name}.npz"))
    so, p, ncrit, theta = int(g["source_order"]), int(g["order"]), int(g["ncrit"]), float(g["theta"])
    t = fg.build_tree(g["pos"], g["S"], len(g["pos"]), ncrit, p, theta, source_order=so)
    F = t.compute_field_bh().cpu().numpy()
    assert rel(F[:, 0], g["phi"]) < 1e-11
    Fo = oracle_lib.OracleTree(g["pos"], g["S"], ncrit, p, theta, so).evaluate_bh()
    assert rel(F[:, 1:], Fo[:, 1:]) < 1e-11


def test_bh_output_switches(fg):
    rng = np.random.default_rng(5)
    n = 4000
    pos, S = rng.uniform(0, 1, (n, 3)), rng.uniform(-1, 1, (n, 1))
    t = fg.build_tree(pos, S, n, 32, 5, 0.5)
    F = t.compute_field_bh().cpu().numpy()
    assert np.array_equal(t.compute_field_bh(potential=True, field=False).cpu().numpy()[:, 0], F[:, 0])
    assert np.array_equal(t.compute_field_bh(potential=False, field=True).cpu().numpy(), F[:, 1:])
    # host output arrays work as for the FMM
    Fh = np.zeros((n, 4))
    t.compute_field_bh(Fh)
    assert np.array_equal(Fh, F)


def test_bh_converges_with_order(fg):
    rng = np.random.default_rng(6)
    n = 20000
    pos = torch.tensor(rng.uniform(0, 1, (n, 3)), device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (n, 1)), device="cuda")
    tg = np.arange(0, n, 20)
    Fd = fg.direct(pos, S, targets=tg).cpu().numpy()
    err = []
    for p in (2, 4, 6, 8):
        F = fg.build_tree(pos, S, n, 64, p, 0.5).compute_field_bh().cpu().numpy()
        err.append(rel(F[tg, 1:], Fd[:, 1:]))
    assert err[0] > err[1] > err[2] > err[3], err


def test_bh_forest_matches_separate_trees(fg):
    rng = np.random.default_rng(7)
    sizes = [700, 3000, 37, 1500]
    pos = np.concatenate([rng.uniform(0, 1, (k, 3)) * (1 + i) + i for i, k in enumerate(sizes)])
    S = rng.uniform(-1, 1, (sum(sizes), 1))
    f = fg.build_forest(torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda"), sizes, 32, 5, 0.5)
    F = f.compute_field_bh().cpu().numpy()
    off = np.concatenate([[0], np.cumsum(sizes)])
    for s, k in enumerate(sizes):
        sl = slice(off[s], off[s + 1])
        G = fg.build_tree(pos[sl], S[sl], k, 32, 5, 0.5).compute_field_bh().cpu().numpy()
        assert rel(F[sl], G) < 1e-13


def test_m2p_operator(fg, oracle_lib):
    """M2P on the operator surface: the batched device call, the scalar twin and
    the module method against the reference's M2P potential and the oracle's
    field."""
    from fmmgen_gb300 import operators

    g = np.load(os.path.join(GOLDEN, "m2p_potential.npz"))
    for so, (pmin, pmax) in ((0, (1, 8)), (1, (2, 6))):
        for p in range(pmin, pmax + 1):
            d, M, phi = g[f"so{so}_p{p}_d"], g[f"so{so}_p{p}_M"], g[f"so{so}_p{p}_phi"]
            K = len(d)
            F = torch.zeros((K, 4), dtype=torch.float64, device="cuda")
            operators.M2P_batch(torch.tensor(d, device="cuda"), torch.tensor(M, device="cuda"), F, p, so)
            F = F.cpu().numpy()
            Fo = np.zeros((K, 4))
            for k in range(K):
                oracle_lib.M2P(*d[k], np.ascontiguousarray(M[k]), Fo[k], p, so)
            assert np.allclose(F[:, 0], phi, rtol=1e-12, atol=0)
            assert np.allclose(F[:, 1:], Fo[:, 1:], rtol=1e-11, atol=1e-14 * np.abs(Fo).max())
            mod = operators.module(pmax + 1, source_order=so)
            Fs = np.zeros(4)
            mod.M2P(*d[0], np.ascontiguousarray(M[0]), Fs, p)
            getattr(mod, f"M2P{p}")(*d[0], np.ascontiguousarray(M[0]), Fs)  # += semantics: twice
            assert np.allclose(Fs, 2 * F[0], rtol=1e-12, atol=0)
