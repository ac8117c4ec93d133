"""Forests of independent systems (one handle, one pass): every system must get
exactly the root cube, cells and interaction lists build_tree gives it alone,
and the same fields."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    nb = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / nb) if nb > 0 else float(np.linalg.norm(a))  # a lone particle: F = 0


def make_systems(seed, sizes, so=0):
    rng = np.random.default_rng(seed)
    pos, S = [], []
    for k, n in enumerate(sizes):
        if k % 3 == 0:  # a shifted, scaled uniform cube
            p = rng.uniform(0, 1, (n, 3)) * rng.uniform(0.5, 4.0) + rng.uniform(-2, 2, 3)
        elif k % 3 == 1:  # a few tight clusters
            c = rng.uniform(0, 1, (4, 3))
            p = c[rng.integers(0, 4, n)] + 0.02 * rng.standard_normal((n, 3))
        else:  # a Plummer-like core
            v = rng.standard_normal((n, 3))
            r = 0.1 / np.sqrt(rng.uniform(0.05, 1.0, n) ** (-2.0 / 3.0) - 1.0)
            p = v / np.linalg.norm(v, axis=1, keepdims=True) * r[:, None]
        pos.append(p)
        S.append(rng.uniform(-1, 1, (n, 1)) if so == 0 else rng.standard_normal((n, 3)))
    return pos, S


def check_forest(fg, sizes, p, so, ncrit, seed):
    pos, S = make_systems(seed, sizes, so)
    P = torch.tensor(np.concatenate(pos), device="cuda")
    Sv = torch.tensor(np.concatenate(S), device="cuda")
    f = fg.build_forest(P, Sv, sizes, ncrit, p, 0.5, source_order=so)
    roots, csys = f.systems()
    cells = f.cells()
    F64 = f.compute_field_fmm(precision="fp64").cpu().numpy()
    Fmx = f.compute_field_fmm(precision="mixed").cpu().numpy()
    f.times()
    off = np.concatenate([[0], np.cumsum(sizes)])
    tot = dict(nm2l=0, np2p=0, inter=0, ncells=0)
    for s, n in enumerate(sizes):
        t = fg.build_tree(torch.tensor(pos[s], device="cuda"), torch.tensor(S[s], device="cuda"), n, ncrit, p, 0.5,
                          source_order=so)
        assert np.array_equal(roots[s], t.root())
        tc = t.cells()
        mine = csys == s
        assert np.array_equal(cells["id"][mine], tc["id"])
        assert np.array_equal(cells["centre"][mine], tc["centre"])
        assert np.array_equal(cells["count"][mine], tc["count"])
        tot["nm2l"] += t.nm2l
        tot["np2p"] += t.np2p
        tot["inter"] += t.p2p_interactions
        tot["ncells"] += t.ncells
        G64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
        Gmx = t.compute_field_fmm(precision="mixed").cpu().numpy()
        sl = slice(off[s], off[s + 1])
        # the same pairs; only the order of M2L terms differs (class ids are ranks over the forest's classes)
        assert rel(F64[sl], G64) < 1e-12
        assert rel(Fmx[sl], Gmx) < 1e-6
    assert (f.nm2l, f.np2p, f.p2p_interactions, f.ncells) == (tot["nm2l"], tot["np2p"], tot["inter"],
                                                              tot["ncells"])


@pytest.mark.parametrize("p,so,ncrit", [(6, 0, 32), (5, 1, 16), (8, 0, 64)])
def test_forest_matches_separate_trees(fg, p, so, ncrit):
    sizes = [1000, 37, 5000, 257, 1, 2048, 300, 4096, 12]
    check_forest(fg, sizes, p, so, ncrit, 5 + p)


def test_forest_of_one_is_a_tree(fg):
    rng = np.random.default_rng(3)
    n = 20000
    P = torch.tensor(rng.uniform(0, 1, (n, 3)), device="cuda")
    Sv = torch.tensor(rng.uniform(-1, 1, (n, 1)), device="cuda")
    f = fg.build_forest(P, Sv, [n], 64, 8, 0.5)
    t = fg.build_tree(P, Sv, n, 64, 8, 0.5)
    for prec in ("fp64", "mixed"):
        assert np.array_equal(f.compute_field_fmm(precision=prec).cpu().numpy(),
                              t.compute_field_fmm(precision=prec).cpu().numpy())


def test_forest_rejects_empty_systems(fg):
    P = torch.zeros((10, 3), dtype=torch.float64, device="cuda")
    Sv = torch.ones((10, 1), dtype=torch.float64, device="cuda")
    with pytest.raises(ValueError):
        fg.build_forest(P, Sv, [5, 0, 5])
