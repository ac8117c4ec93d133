"""The CPU checker (oracle/) pinned against the reference: golden vectors written
by the reference's own generated operators and tree code (tests/golden), and the
known answers of the reference's unit tests."""
import os

import numpy as np
import pytest

from conftest import GOLDEN


def relerr(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-300)


def test_index_layout(oracle_lib):
    # fmmgen/utils.py:65-118 ordering: degree, then nx desc, then ny desc
    expect = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 0, 0), (1, 1, 0), (1, 0, 1), (0, 2, 0), (0, 1, 1),
              (0, 0, 2), (3, 0, 0), (2, 1, 0), (2, 0, 1), (1, 2, 0), (1, 1, 1), (1, 0, 2), (0, 3, 0), (0, 2, 1),
              (0, 1, 2), (0, 0, 3)]
    for i, n in enumerate(expect):
        assert oracle_lib.lib().or_index(*n) == i
    assert [oracle_lib.nterms(p) for p in (4, 6, 8, 12)] == [35, 84, 165, 455]
    assert oracle_lib.msize(6, 1) == 83 and oracle_lib.lsize(6, 1) == 56


@pytest.mark.parametrize("so", [0, 1, 2])
def test_operators_match_generated(oracle_lib, so):
    """Every operator at every generated order vs fmmgen's generated C (1e-12)."""
    g = np.load(os.path.join(GOLDEN, f"ops_so{so}.npz"))
    O = oracle_lib
    for p in range(int(g["pmin"]), int(g["pmax"]) + 1):
        d, q, Min, Lin = g[f"p{p}_d"], g[f"p{p}_q"], g[f"p{p}_M"], g[f"p{p}_L"]
        ms, ls = O.msize(p, so), O.lsize(p, so)
        for i in range(len(d)):
            a = np.zeros(ms); O.P2M(*d[i], q[i], a, p, so)
            assert relerr(a, g[f"p{p}_P2M"][i]) < 1e-12
            a = np.zeros(ms); O.M2M(*d[i], Min[i].copy(), a, p, so)
            assert relerr(a, g[f"p{p}_M2M"][i]) < 1e-12
            a = np.zeros(ls); O.M2L(*d[i], Min[i].copy(), a, p, so)
            assert relerr(a, g[f"p{p}_M2L"][i]) < 1e-12, (p, i)
            a = np.zeros(ls); O.L2L(*d[i], Lin[i].copy(), a, p, so)
            assert relerr(a, g[f"p{p}_L2L"][i]) < 1e-12
            a = np.zeros(4); O.L2P(*d[i], Lin[i].copy(), a, p, so)
            assert relerr(a, g[f"p{p}_L2P"][i]) < 1e-12


@pytest.mark.parametrize("so", [0, 1, 2])
def test_p2p_restated(oracle_lib, so):
    g = np.load(os.path.join(GOLDEN, f"ops_so{so}.npz"))
    for i in range(len(g["p2p_d"])):
        F = np.zeros(4)
        oracle_lib.P2P(*g["p2p_d"][i], g["p2p_S"][i].copy(), F, so)
        assert relerr(F, g["p2p_F"][i]) < 1e-14
    # the generated P2P agrees on the potential; its field is what fmmgen at HEAD gets wrong
    assert np.allclose(g["p2p_F"][:, 0], g["p2p_F_generated"][:, 0], rtol=1e-13)
    if so == 0:
        assert np.all(g["p2p_F_generated"][:, 1:] == 0)


@pytest.mark.parametrize("so", [0, 1, 2])
def test_float_fixtures_are_float_rounding(so):
    """ops_f32_so*.npz (the reference's precision="float" operators) sit within
    float rounding of the FP64 generated operators on the same inputs, so they
    measure the FP32 variant's accuracy and nothing else."""
    g = np.load(os.path.join(GOLDEN, f"ops_so{so}.npz"))
    f = np.load(os.path.join(GOLDEN, f"ops_f32_so{so}.npz"))
    for p in range(int(g["pmin"]), int(g["pmax"]) + 1):
        for k in ("P2M", "M2M", "M2L", "L2L", "L2P"):
            a, b = f[f"p{p}_{k}"], g[f"p{p}_{k}"]
            assert a.dtype == np.float32 and a.shape == b.shape
            assert np.all(np.max(np.abs(a - b), axis=1) <= 2e-5 * np.max(np.abs(b), axis=1)), (p, k)
    assert relerr(f["p2p_phi"], g["p2p_F"][:, 0]) < 1e-6


def test_reference_known_answers(oracle_lib):
    """The numeric assertions of the reference's tests/test_multipoles.py."""
    O = oracle_lib
    for order in range(1, 4):  # test_linear_dipole (tests/test_multipoles.py:11-65)
        d, q = 1.0, 5.0
        M = np.zeros(O.nterms(order))
        for x, s in ((np.array([d, 0, 0]), q), (np.array([-d, 0, 0]), -q)):
            S = np.zeros(O.nterms(order)); S[0] = s
            O.M2M(*(-x), S, M, order)
        assert M[0] == 0.0 and M[1] == -2 * q * d and M[2] == 0.0 and M[3] == 0.0
    for order in range(2, 4):  # test_linear_quadrupole (:68-133)
        d, q = 2.0, 5.0
        M = np.zeros(O.nterms(order))
        for x, s in ((np.array([-d, 0, 0]), -q), (np.array([d, 0, 0]), -q), (np.zeros(3), 2 * q)):
            S = np.zeros(O.nterms(order)); S[0] = s
            O.M2M(*(-x), S, M, order)
        assert M[0] == 0.0 and M[1] == 0.0 and M[2] == 0.0 and M[3] == 0.0 and M[4] == -2 * d * q
    for order in range(2, 4):  # test_quadrupole_two_dipoles (:136-197)
        d, mux = 2.0, -5.0
        M = np.zeros(O.nterms(order))
        for x, s in ((np.array([d, 0, 0]), -mux), (np.array([-d, 0, 0]), mux)):
            S = np.zeros(O.nterms(order)); S[1] = s
            O.M2M(*(-x), S, M, order)
        assert M[0] == 0.0 and M[1] == 0.0 and M[2] == 0.0 and M[3] == 0.0 and M[4] == 2 * mux * d


TREES = ["uniform10k", "deep", "dipole_plummer", "clustered", "tiny", "example_scaled", "quadrupole_plummer"]


def canonical(pairs):
    a = np.ascontiguousarray(pairs, dtype=np.uint64).reshape(-1, 2)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def leaf_sets(ids, off, idx):
    return {int(i): tuple(sorted(idx[off[k]:off[k + 1]].tolist())) for k, i in enumerate(ids)}


@pytest.mark.parametrize("case", TREES)
def test_tree_matches_reference(oracle_lib, case):
    import hashlib

    g = np.load(os.path.join(GOLDEN, f"tree_{case}.npz"))
    so = int(g["source_order"])
    t = oracle_lib.OracleTree(g["pos"], g["S"], int(g["ncrit"]), int(g["order"]), float(g["theta"]), so)
    c = t.cells()
    o = np.argsort(c["id"])
    assert np.array_equal(c["id"][o], g["cell_id"])
    assert np.array_equal(c["nleaf"][o], g["cell_nleaf"])
    assert np.array_equal(c["centre"][o], g["cell_centre"])  # bit-exact FP64 centres
    mine = leaf_sets(c["id"][c["leaf_cell"]], c["leaf_off"], c["leaf_idx"])
    ref = leaf_sets(g["leaf_id"], g["leaf_off"], g["leaf_idx"])
    assert mine == ref
    m2l, p2p = t.lists()
    assert len(m2l) == int(g["nm2l"]) and len(p2p) == int(g["np2p"])
    assert hashlib.sha256(canonical(m2l).tobytes()).hexdigest() == str(g["m2l_sha256"])
    assert hashlib.sha256(canonical(p2p).tobytes()).hexdigest() == str(g["p2p_sha256"])
    F, _ = t.evaluate()
    assert np.linalg.norm(F - g["F"]) <= 1e-13 * np.linalg.norm(g["F"])


def test_fmm_accuracy_vs_direct(oracle_lib):
    g = np.load(os.path.join(GOLDEN, "tree_uniform10k.npz"))
    t = oracle_lib.OracleTree(g["pos"], g["S"], 64, 4, 0.5, 0)
    F, _ = t.evaluate()
    idx = np.arange(0, 10000, 7)
    Fd = oracle_lib.direct(g["pos"], g["S"], idx)
    e = np.linalg.norm(F[idx, 1:] - Fd[:, 1:]) / np.linalg.norm(Fd[:, 1:])
    assert 1e-5 < e < 5e-4  # p=4, theta=0.5 truncation error


def test_quadrupole_p2p_is_the_field_of_its_potential(oracle_lib):
    """Quadrupole sources (source_order 2): the restated P2P field is minus the
    gradient of the potential the generated P2P gives (central differences)."""
    g = np.load(os.path.join(GOLDEN, "ops_so2.npz"))
    h = 1e-6
    for i in range(len(g["p2p_d"])):
        d, S = g["p2p_d"][i], g["p2p_S"][i]
        grad = []
        for a in range(3):
            e = np.zeros(3); e[a] = h
            Fp, Fm = np.zeros(4), np.zeros(4)
            oracle_lib.P2P(*(d + e), S.copy(), Fp, 2)
            oracle_lib.P2P(*(d - e), S.copy(), Fm, 2)
            grad.append(-(Fp[0] - Fm[0]) / (2 * h))
        assert relerr(grad, g["p2p_F"][i][1:]) < 1e-7


def test_oracle_rejects_coincident_points(oracle_lib):
    pos = np.zeros((100, 3))
    with pytest.raises(ValueError):
        oracle_lib.OracleTree(pos, np.ones((100, 1)), 8, 3, 0.5, 0)


def test_exact_target_subset_equals_full_pass(oracle_lib):
    """sample_stride < -1: the fields of every k-th leaf's particles equal the
    full pass's bit for bit (M2L into their ancestors too), other rows zero."""
    rng = np.random.default_rng(31)
    pos = rng.uniform(0, 1, (20000, 3))
    q = rng.uniform(-1, 1, (20000, 1))
    ot = oracle_lib.OracleTree(pos, q, 32, 4, 0.5, 0)
    Ff, _ = ot.evaluate()
    Fs, _ = ot.evaluate(sample_stride=-7)
    rows = np.any(Fs != 0.0, axis=1)
    assert 1000 < rows.sum() < 6000
    assert np.array_equal(Fs[rows], Ff[rows])
