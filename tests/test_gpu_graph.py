"""Graph mode: the evaluation pass recorded once as a CUDA graph and replayed
must give exactly the fields of a normal pass, follow rebuilds and argument
changes, and count its kernels."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def data(seed, n, so=0):
    rng = np.random.default_rng(seed)
    pos = torch.tensor(rng.uniform(0, 1, (n, 3)), device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (n, 1)) if so == 0 else rng.standard_normal((n, 3)), device="cuda")
    return pos, S


@pytest.mark.parametrize("precision", ["mixed", "fp64", "mixed_simt"])
def test_graph_replay_matches(fg, precision):
    pos, S = data(1, 40000)
    plain = fg.build_tree(pos, S, 40000, 64, 6, 0.5)
    ref = plain.compute_field_fmm(precision=precision).cpu().numpy()
    t = fg.build_tree(pos, S, 40000, 64, 6, 0.5).set_graph(True)
    F = torch.empty((40000, 4), dtype=torch.float64, device="cuda")
    L = fg.lib()
    n0 = L.fmmgen_launch_count()
    t.compute_field_fmm(F, precision=precision)  # normal pass, then recorded
    first = L.fmmgen_launch_count() - n0
    assert np.array_equal(F.cpu().numpy(), ref)
    counts = []
    for _ in range(3):
        F.zero_()
        n0 = L.fmmgen_launch_count()
        t.compute_field_fmm(F, precision=precision)  # replays
        counts.append(L.fmmgen_launch_count() - n0)
        assert np.array_equal(F.cpu().numpy(), ref)
    # each replay counts the graph's kernels; the first pass after a build may
    # also have built the per-build tensor-core operator records
    assert counts[0] == counts[1] == counts[2] and 0 < counts[0] <= first
    b, e = t.times()
    assert e["total"] > 0 and e["M2L"] > 0  # the replayed pass records its phase times


def test_graph_follows_rebuild_and_arguments(fg):
    pos, S = data(2, 30000)
    pos2, S2 = data(3, 30000)
    t = fg.build_tree(pos, S, 30000, 32, 5, 0.5).set_graph(True)
    t.compute_field_fmm(precision="mixed")
    t.compute_field_fmm(precision="mixed")
    # new sources: a new recording
    got = t.compute_field_fmm(S=S2, precision="mixed").cpu().numpy()
    ref = fg.build_tree(pos, S2, 30000, 32, 5, 0.5).compute_field_fmm(precision="mixed").cpu().numpy()
    assert np.array_equal(got, ref)
    # new positions: a new build, so a new recording
    t.rebuild(pos2)
    got = [t.compute_field_fmm(S=S2, precision="mixed").cpu().numpy() for _ in range(2)]
    ref = fg.build_tree(pos2, S2, 30000, 32, 5, 0.5).compute_field_fmm(precision="mixed").cpu().numpy()
    assert np.array_equal(got[0], ref) and np.array_equal(got[1], ref)
    t.set_graph(False)
    assert np.array_equal(t.compute_field_fmm(S=S2, precision="mixed").cpu().numpy(), ref)


def test_graph_forest(fg):
    sizes = [3000, 500, 12000, 7]
    pos, S = data(4, sum(sizes))
    f = fg.build_forest(pos, S, sizes, 32, 6, 0.5)
    ref = f.compute_field_fmm(precision="mixed").cpu().numpy()
    f.set_graph(True)
    for _ in range(3):
        assert np.array_equal(f.compute_field_fmm(precision="mixed").cpu().numpy(), ref)
    f.times()
