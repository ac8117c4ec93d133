"""Device octree + interaction lists, bit-exact against the reference's
build_tree / interact_dehnen_lazy (golden fixtures) and the CPU restatement."""
import hashlib
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
TREES = ["uniform10k", "deep", "dipole_plummer", "clustered", "tiny", "example_scaled"]


def canonical(pairs):
    a = np.ascontiguousarray(pairs, dtype=np.uint64).reshape(-1, 2)
    return a[np.lexsort((a[:, 1], a[:, 0]))]


def leaf_sets(ids, off, idx):
    return {int(i): tuple(sorted(idx[off[k]:off[k + 1]].tolist())) for k, i in enumerate(ids)}


def gpu_tree(fg, g):
    pos = torch.tensor(g["pos"], device="cuda")
    S = torch.tensor(g["S"], device="cuda")
    return fg.build_tree(pos, S, int(g["N"]), int(g["ncrit"]), int(g["order"]), float(g["theta"]),
                         source_order=int(g["source_order"]))


def check_against(t, cell_id, cell_count, centre, leaf_id, leaf_off, leaf_idx, m2l_digest, p2p_digest, nm2l, np2p,
                  m2l=None, p2p=None):
    c = t.cells()
    o = np.argsort(c["id"])
    assert np.array_equal(c["id"][o], cell_id)
    assert np.array_equal(c["count"][o], cell_count)
    assert np.array_equal(c["centre"][o], centre)  # bit-exact FP64 centres
    ncrit = t.ncrit
    leaf_ids = c["id"][c["count"] < ncrit]
    assert leaf_sets(leaf_ids, c["leaf_off"], c["leaf_idx"]) == leaf_sets(leaf_id, leaf_off, leaf_idx)
    gm, gp = t.lists()
    assert (len(gm), len(gp)) == (nm2l, np2p)
    cm, cp = canonical(gm), canonical(gp)
    assert hashlib.sha256(cm.tobytes()).hexdigest() == m2l_digest
    assert hashlib.sha256(cp.tobytes()).hexdigest() == p2p_digest
    if m2l is not None:
        assert np.array_equal(cm, m2l) and np.array_equal(cp, p2p)


@pytest.mark.parametrize("case", TREES)
def test_tree_bit_exact_vs_reference(fg, case):
    g = np.load(os.path.join(GOLDEN, f"tree_{case}.npz"))
    t = gpu_tree(fg, g)
    check_against(t, g["cell_id"], g["cell_nleaf"], g["cell_centre"], g["leaf_id"], g["leaf_off"], g["leaf_idx"],
                  str(g["m2l_sha256"]), str(g["p2p_sha256"]), int(g["nm2l"]), int(g["np2p"]),
                  g["m2l"] if "m2l" in g else None, g["p2p"] if "p2p" in g else None)


def oracle_check(fg, oracle_lib, pos, S, ncrit, p, theta, so=0):
    ot = oracle_lib.OracleTree(pos, S, ncrit, p, theta, so)
    oc = ot.cells()
    o = np.argsort(oc["id"])
    om, op = ot.lists()
    t = fg.build_tree(torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda"), len(pos), ncrit, p, theta,
                      source_order=so)
    check_against(t, oc["id"][o], oc["nleaf"][o], oc["centre"][o], oc["id"][oc["leaf_cell"]], oc["leaf_off"],
                  oc["leaf_idx"], hashlib.sha256(canonical(om).tobytes()).hexdigest(),
                  hashlib.sha256(canonical(op).tobytes()).hexdigest(), len(om), len(op))
    return t, ot


@pytest.mark.parametrize("N,ncrit,theta,seed", [(20000, 32, 0.5, 11), (50000, 128, 0.5, 12), (8000, 4, 0.3, 13),
                                                  (30000, 64, 0.8, 14), (1000, 2, 0.5, 15), (64, 64, 0.5, 16),
                                                  (65, 64, 0.5, 17)])
def test_tree_vs_checker_random(fg, oracle_lib, N, ncrit, theta, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 1, (N, 3))
    oracle_check(fg, oracle_lib, pos, rng.uniform(-1, 1, (N, 1)), ncrit, 4, theta)


def test_tree_points_on_split_planes(fg, oracle_lib):
    """Points on a grid lattice sit exactly on cell planes (strict > test)."""
    g = np.arange(16) / 15.0
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(3)
    oracle_check(fg, oracle_lib, pos, rng.uniform(-1, 1, (len(pos), 1)), 16, 3, 0.5)


def test_tree_strongly_clustered(fg, oracle_lib):
    rng = np.random.default_rng(5)
    pos = np.concatenate([0.5 + 1e-4 * rng.standard_normal((4000, 3)), rng.uniform(0, 1, (4000, 3))])
    oracle_check(fg, oracle_lib, pos, rng.uniform(-1, 1, (8000, 1)), 16, 4, 0.5)


@pytest.mark.parametrize("dist", ["offset", "negative", "unit_1m", "centred", "dyadic_ties", "tiny_scale", "single"])
def test_root_box_bits(fg, oracle_lib, dist):
    """Sequential-sum mean and 1.001 * max |x - mean| exactly as build_tree."""
    rng = np.random.default_rng(9)
    n = 1_000_000 if dist == "unit_1m" else 123457
    if dist == "offset":
        pos = rng.uniform(-3, 7, (n, 3))
    elif dist == "negative":  # negative running sums across binades
        pos = rng.uniform(-7, 2, (n, 3))
    elif dist == "unit_1m":  # long runs of chunks inside one binade
        pos = rng.uniform(0, 1, (n, 3))
    elif dist == "centred":  # running sums wander across binades around zero
        pos = 0.1 * rng.standard_normal((n, 3))
    elif dist == "dyadic_ties":  # short mantissas: many additions round half-way
        pos = np.round(rng.uniform(0, 1, (n, 3)) * 2 ** 20) / 2 ** 21 + 0.5
    elif dist == "tiny_scale":  # the example driver's scaling (example/main.cpp:86-110)
        pos = rng.uniform(-1, 1, (n, 3)) * 1e-9
    else:
        pos = rng.uniform(0, 1, (1, 3))
    t = fg.build_tree(torch.tensor(pos, device="cuda"), torch.ones(len(pos), 1, dtype=torch.float64, device="cuda"),
                      len(pos), 64, 3, 0.5)
    r = t.root()
    s = np.zeros(3)
    for k in range(3):  # the reference's sequential loop (example/tree.cpp:148-156)
        acc = 0.0
        for v in pos[:, k].tolist():
            acc += v
        s[k] = acc / len(pos)
    assert np.array_equal(r[:3], s)
    m = max(np.max(np.abs(pos[:, k] - s[k])) for k in range(3)) * 1.001
    assert r[3] == m


def test_error_codes(fg):
    from fmmgen_gb300 import FMMError, _lib

    dup = torch.zeros(200, 3, dtype=torch.float64, device="cuda")
    with pytest.raises(FMMError) as e:
        fg.build_tree(dup, torch.ones(200, 1, dtype=torch.float64, device="cuda"), 200, 16, 4, 0.5)
    assert e.value.code == _lib.ERR_DEPTH
    # fewer coincident points than ncrit is a single leaf and evaluates
    t = fg.build_tree(dup[:10], torch.ones(10, 1, dtype=torch.float64, device="cuda"), 10, 16, 4, 0.5)
    assert t.ncells == 1 and t.np2p == 1
    with pytest.raises(FMMError):
        fg.build_tree(dup[:10], torch.ones(10, 1, dtype=torch.float64, device="cuda"), 10, 16, 13, 0.5)


def test_handle_reuse(fg, oracle_lib):
    """A rebuilt handle (new positions, reused buffers) equals a fresh build."""
    rng = np.random.default_rng(21)
    a = rng.uniform(0, 1, (30000, 3))
    b = rng.uniform(0, 1, (12000, 3))
    q = rng.uniform(-1, 1, (30000, 1))
    t = fg.build_tree(torch.tensor(a, device="cuda"), torch.tensor(q, device="cuda"), 30000, 64, 4, 0.5)
    t.rebuild(torch.tensor(b, device="cuda"))
    t2 = fg.build_tree(torch.tensor(b, device="cuda"), torch.tensor(q[:12000], device="cuda"), 12000, 64, 4, 0.5)
    assert (t.ncells, t.nm2l, t.np2p) == (t2.ncells, t2.nm2l, t2.np2p)
    assert all(np.array_equal(x, y) for x, y in zip(t.lists(), t2.lists()))
