"""rebuild_compute (fmmgen_tree_build_compute): the build and the evaluation in
one call, the near field and the multipoles computed while the build groups
the M2L lists.  It must give exactly the fields of rebuild + compute_field_fmm,
for one tree, a forest, every precision, learned orders and the tuned M2L
choices, and report the build's errors."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def system(seed, n, so=0):
    rng = np.random.default_rng(seed)
    pos = torch.tensor(rng.uniform(0, 1, (n, 3)), device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (n, 1)) if so == 0 else rng.standard_normal((n, 3)), device="cuda")
    return pos, S


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_simt"])
@pytest.mark.parametrize("so,p", [(0, 8), (1, 6)])
def test_fused_equals_two_calls(fg, precision, so, p):
    n = 30000
    pos, S = system(1 + p, n, so)
    pos2, _ = system(2 + p, n, so)
    a = fg.build_tree(pos, S, n, 64, p, 0.5, source_order=so)
    b = fg.build_tree(pos, S, n, 64, p, 0.5, source_order=so)
    for P in (pos2, pos):
        a.rebuild(P)
        Fa = a.compute_field_fmm(precision=precision).cpu().numpy()
        Fb = b.rebuild_compute(P, precision=precision).cpu().numpy()
        assert np.array_equal(Fa, Fb)
        assert (a.ncells, a.nm2l, a.np2p, a.nclasses) == (b.ncells, b.nm2l, b.np2p, b.nclasses)
    b.times()  # phase records of the fused pass are readable


@pytest.mark.parametrize("overlap", [0, 2])
def test_fused_with_tuning_and_learned_orders(fg, overlap):
    from fmmgen_gb300 import learned

    n = 40000
    pos, S = system(5, n)
    a = fg.build_tree(pos, S, n, 64, 8, 0.5).set_tune(0, 3, 0, overlap)
    b = fg.build_tree(pos, S, n, 64, 8, 0.5).set_tune(0, 3, 0, overlap)
    assert np.array_equal(a.compute_field_fmm(precision="mixed").cpu().numpy(),
                          b.rebuild_compute(pos, precision="mixed").cpu().numpy())
    m = learned.OrderModel.load()
    m.attach(a)
    m.attach(b)
    Fa = a.compute_field_fmm(precision="mixed").cpu().numpy()
    Fb = b.rebuild_compute(pos, precision="mixed").cpu().numpy()
    assert np.array_equal(Fa, Fb) and np.array_equal(a.m2l_orders(), b.m2l_orders())


@pytest.mark.parametrize("so,overlap", [(0, 0), (0, 2), (1, 2)])
def test_fused_forest(fg, so, overlap):
    sizes = [3000, 40, 12000, 700]
    rng = np.random.default_rng(9)
    pos = torch.tensor(np.concatenate([rng.uniform(0, 1, (k, 3)) + 2 * i for i, k in enumerate(sizes)]),
                       device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (sum(sizes), 1 if so == 0 else 3)), device="cuda")
    a = fg.build_forest(pos, S, sizes, 32, 6, 0.5, source_order=so).set_tune(0, 0, 0, overlap)
    b = fg.build_forest(pos, S, sizes, 32, 6, 0.5, source_order=so).set_tune(0, 0, 0, overlap)
    c = fg.build_forest(pos, S, sizes, 32, 6, 0.5, source_order=so)  # default choices, separate calls
    Fa = a.compute_field_fmm(precision="mixed").cpu().numpy()
    assert np.array_equal(Fa, b.rebuild_compute(pos, precision="mixed").cpu().numpy())
    assert np.array_equal(Fa, c.compute_field_fmm(precision="mixed").cpu().numpy())


def test_fused_reports_build_errors(fg):
    n = 200
    pos = torch.zeros((n, 3), dtype=torch.float64, device="cuda")  # all coincident: >= ncrit at every level
    S = torch.ones((n, 1), dtype=torch.float64, device="cuda")
    t = fg.build_tree(torch.rand((n, 3), dtype=torch.float64, device="cuda"), S, n, 16, 4, 0.5)
    with pytest.raises(fg.FMMError):
        t.rebuild_compute(pos, precision="mixed")
