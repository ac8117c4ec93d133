"""Barnes-Hut on the CPU: the oracle's M2P and compute_field_bh against the
reference's own potentials (tests/golden/bh_*.npz, m2p_potential.npz), and the
M2P field against the gradient of the M2P potential."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

CASES = ["uniform10k", "clustered", "dipole_plummer"]


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_m2p_potential_matches_reference(oracle_lib):
    g = np.load(os.path.join(GOLDEN, "m2p_potential.npz"))
    checked = 0
    for so, (pmin, pmax) in ((0, (1, 8)), (1, (2, 6))):
        for p in range(pmin, pmax + 1):
            d, M, phi = g[f"so{so}_p{p}_d"], g[f"so{so}_p{p}_M"], g[f"so{so}_p{p}_phi"]
            for k in range(len(d)):
                F = np.zeros(4)
                oracle_lib.M2P(*d[k], np.ascontiguousarray(M[k]), F, p, so)
                assert abs(F[0] - phi[k]) <= 1e-13 * max(1.0, abs(phi[k])), (so, p, k)
                checked += 1
    assert checked == 65


@pytest.mark.parametrize("so,p", [(0, 3), (0, 8), (1, 4)])
def test_m2p_field_is_the_gradient(oracle_lib, so, p):
    rng = np.random.default_rng(p)
    M = rng.standard_normal(oracle_lib.msize(p, so))
    d = np.array([1.7, -0.4, 1.1])
    F = np.zeros(4)
    oracle_lib.M2P(*d, M, F, p, so)
    h = 1e-5
    for a in range(3):
        e = np.zeros(3)
        e[a] = h
        fp, fm = np.zeros(4), np.zeros(4)
        oracle_lib.M2P(*(d + e), M, fp, p, so)
        oracle_lib.M2P(*(d - e), M, fm, p, so)
        assert abs(F[1 + a] + (fp[0] - fm[0]) / (2 * h)) < 1e-8 * np.abs(F[1:]).max()


@pytest.mark.parametrize("name", CASES)
def test_bh_potential_matches_reference(oracle_lib, name):
    g = np.load(os.path.join(GOLDEN, f"bh_{name}.npz"))
    ot = oracle_lib.OracleTree(g["pos"], g["S"], int(g["ncrit"]), int(g["order"]), float(g["theta"]),
                               int(g["source_order"]))
    F = ot.evaluate_bh()
    assert rel(F[:, 0], g["phi"]) < 1e-12
    # the field is a Barnes-Hut field: close to the direct sum at this order and theta
    n = len(g["pos"])
    tg = np.arange(0, n, max(1, n // 500))
    Fd = oracle_lib.direct(g["pos"], g["S"], tg, int(g["source_order"]))
    assert rel(F[tg, 1:], Fd[:, 1:]) < 2e-2
