"""The M2L autotuner: every candidate it times is a valid M2L (fields within
the mixed-precision tolerance of the FP64 pass), the handle keeps the fastest,
explicit settings are honoured or rejected, and graph replays follow them."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def system(seed, n, so=0):
    rng = np.random.default_rng(seed)
    pos = torch.tensor(rng.uniform(0, 1, (n, 3)), device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (n, 1)) if so == 0 else rng.standard_normal((n, 3)), device="cuda")
    return pos, S


@pytest.mark.parametrize("p,so", [(8, 0), (6, 1), (10, 0)])
def test_autotune_candidates(fg, p, so):
    n = 60000
    pos, S = system(3 + p, n, so)
    t = fg.build_tree(pos, S, n, 64, p, 0.5, source_order=so)
    ref = t.compute_field_fmm(precision="fp64").cpu().numpy()
    r = t.autotune(precision="mixed", reps=2)
    table = r["table"]
    impls = {c["impl"] for c in table}
    assert 2 in impls and {c["grouping"] for c in table} == {0, 1}
    assert (0 in impls) == (p <= 9)  # tensor cores where the order allows
    assert all(c["ms"] > 0 for c in table)
    best = min(table, key=lambda c: c["ms"])
    key = ("impl", "nslots", "grouping", "overlap")
    if r["best"] != {k: best[k] for k in key}:
        # the serial twin of an overlapped fastest candidate, within 2 % of it
        assert best["overlap"] and r["best"]["overlap"] == 0, (r["best"], best)
        twin = [c for c in table if {k: c[k] for k in key} == r["best"]]
        assert twin and all(r["best"][k] == best[k] for k in key[:3]) and twin[0]["ms"] <= 1.02 * best["ms"]
    F = t.compute_field_fmm(precision="mixed").cpu().numpy()
    assert rel(F, ref) < 2e-6
    for c in table:
        t.set_tune(c["impl"], c["nslots"], c["grouping"], c["overlap"])
        assert rel(t.compute_field_fmm(precision="mixed").cpu().numpy(), ref) < 2e-6, c


def test_pipeline_depth_does_not_change_results(fg):
    n = 50000
    pos, S = system(11, n)
    t = fg.build_tree(pos, S, n, 64, 8, 0.5)
    out = []
    for s in (2, 3, 4):
        t.set_tune(0, s, 0)
        out.append(t.compute_field_fmm(precision="mixed").cpu().numpy())
    assert np.array_equal(out[0], out[1]) and np.array_equal(out[0], out[2])


def test_set_tune_rejects_unsupported(fg):
    n = 20000
    pos, S = system(12, n)
    t = fg.build_tree(pos, S, n, 64, 12, 0.5)
    with pytest.raises(fg.FMMError):
        t.set_tune(0)  # no tensor-core M2L at p = 12
    with pytest.raises(fg.FMMError):
        t.set_tune(1)  # no generated kernels at p = 12
    with pytest.raises(fg.FMMError):
        t.set_tune(6)  # no such implementation
    t.set_tune(5)  # the target-major generated kernels cover p = 12
    t.set_tune(2, 0, 1)
    assert t.get_tune() == {"impl": 2, "nslots": 0, "grouping": 1, "overlap": 0}


def test_overlap_gives_the_same_fields(fg):
    n = 80000
    pos, S = system(14, n)
    t = fg.build_tree(pos, S, n, 64, 8, 0.5)
    t.set_tune(0, 0, 0, 0)
    ref = t.compute_field_fmm(precision="mixed").cpu().numpy()
    for ov in (1, 2, 1):
        t.set_tune(0, 0, 0, ov)
        assert np.array_equal(t.compute_field_fmm(precision="mixed").cpu().numpy(), ref)
    b, e = t.times()
    assert e["M2L"] > 0 and e["P2P"] >= 0


def test_tune_under_graph_replay(fg):
    n = 40000
    pos, S = system(13, n)
    t = fg.build_tree(pos, S, n, 64, 8, 0.5).set_graph(True)
    F = torch.empty((n, 4), dtype=torch.float64, device="cuda")
    for impl, grouping, ov in ((0, 0, 0), (1, 1, 0), (0, 1, 1), (0, 0, 2)):
        t.set_tune(impl, 0, grouping, ov)
        ref = fg.build_tree(pos, S, n, 64, 8, 0.5).set_tune(impl, 0, grouping, ov).compute_field_fmm(
            precision="mixed").cpu().numpy()
        for _ in range(2):
            t.compute_field_fmm(F, precision="mixed")
            assert np.array_equal(F.cpu().numpy(), ref)


@pytest.mark.parametrize("p,so", [(12, 0), (7, 1), (5, 2)])
def test_fp32_engine_m2l_vs_fp64(fg, p, so):
    """The FP32 engine M2L (two source cells per packed-FMA pass, an odd last
    pair beside zeros) against the FP64 pass, for each source order."""
    n = 30000
    rng = np.random.default_rng(40 + p)
    pos = torch.tensor(rng.uniform(0, 1, (n, 3)), device="cuda")
    S = torch.tensor(rng.standard_normal((n, {0: 1, 1: 3, 2: 6}[so])), device="cuda")
    t = fg.build_tree(pos, S, n, 64, p, 0.5, source_order=so)
    ref = t.compute_field_fmm(precision="fp64").cpu().numpy()
    t.set_tune(2, 0, 0, 0)
    F = t.compute_field_fmm(precision="mixed").cpu().numpy()
    assert rel(F[:, 1:], ref[:, 1:]) < 5e-6
    assert rel(F[:, 0], ref[:, 0]) < 5e-6
    again = t.compute_field_fmm(precision="mixed").cpu().numpy()
    assert np.array_equal(F, again)
