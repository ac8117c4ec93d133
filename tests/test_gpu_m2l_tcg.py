"""Tensor-core M2L with source rows boxed from dense level grids (impl 3):
on trees whose levels are all complete it must run (m2l_work reports the
boxes), agree with the row-gather tensor-core kernel (impl 0) and the FP64
pass, be deterministic, and fall back to the row gather elsewhere."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def uniform(n, so, seed):
    rng = np.random.default_rng(seed)
    pos = rng.uniform(0, 1, (n, 3))
    S = rng.uniform(-1, 1, (n, 1)) if so == 0 else rng.standard_normal((n, 3))
    return torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda")


# 200,000 uniform particles, ncrit 128: every level-4 cell is a leaf (~49
# particles), so levels 0-4 are complete
@pytest.mark.parametrize("p,so", [(8, 0), (4, 0), (9, 0), (6, 1), (2, 0)])
def test_boxes_vs_gather_and_fp64(fg, p, so):
    pos, S = uniform(200_000, so, 40 + p)
    t = fg.build_tree(pos, S, pos.shape[0], 128, p, 0.5, source_order=so)
    assert t.nlevels == 5 and t.ncells == sum(8 ** l for l in range(5))
    F64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
    _, L64 = t.expansions()
    t.set_tune(impl=3)
    Fb = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.times()  # raises if a pipeline wait timed out
    steps, mmas, flops, boxes = t.m2l_work()
    assert boxes == 1.0 and steps > 0
    _, Lb = t.expansions()
    Fb2 = t.compute_field_fmm(precision="mixed").cpu().numpy()
    assert np.array_equal(Fb, Fb2)  # deterministic
    t.set_tune(impl=0)
    Fg = t.compute_field_fmm(precision="mixed").cpu().numpy()
    assert t.m2l_work()[3] == 0.0
    _, Lg = t.expansions()
    e_b, e_g = rel(Lb, L64), rel(Lg, L64)
    # one power-of-two scale per level instead of one per row: the same few
    # 2^-22 relative product errors
    assert e_b < max(3 * e_g, 1e-6), (e_b, e_g)
    assert rel(Fb[:, -3:], F64[:, -3:]) < 2e-6
    assert rel(Fb[:, 0], F64[:, 0]) < 2e-6
    assert rel(Fg[:, -3:], F64[:, -3:]) < 2e-6


@pytest.mark.parametrize("nslots", [2, 3])
def test_boxes_shallow_pipelines(fg, nslots):
    """Fewer operand slots than producer warps (one producer per slot)."""
    pos, S = uniform(200_000, 0, 77)
    t = fg.build_tree(pos, S, pos.shape[0], 128, 7, 0.5)
    F64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
    t.set_tune(impl=3, nslots=nslots)
    F = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.times()
    assert t.m2l_work()[3] == 1.0
    assert rel(F[:, -3:], F64[:, -3:]) < 2e-6


def test_boxes_fall_back_on_adaptive_tree(fg):
    rng = np.random.default_rng(3)
    r = 0.1 / np.sqrt(rng.uniform(0.01, 1.0, 40000) ** (-2.0 / 3.0) - 1.0)
    v = rng.standard_normal((40000, 3))
    pos = torch.tensor(v / np.linalg.norm(v, axis=1, keepdims=True) * r[:, None], device="cuda")
    S = torch.tensor(rng.uniform(-1, 1, (40000, 1)), device="cuda")
    t = fg.build_tree(pos, S, 40000, 64, 6, 0.5)
    F64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
    t.set_tune(impl=3)
    F = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.times()
    assert t.m2l_work()[3] == 0.0
    assert rel(F[:, -3:], F64[:, -3:]) < 2e-6


def test_boxes_graph_replay_and_rebuild(fg):
    """Recorded as a CUDA graph and replayed, and after a rebuild with new
    positions (new grids, masks and tensor maps), the results match a fresh
    handle bit for bit."""
    pa, S = uniform(200_000, 0, 5)
    pb, _ = uniform(200_000, 0, 6)
    t = fg.build_tree(pa, S, pa.shape[0], 128, 8, 0.5)
    t.set_tune(impl=3)
    t.set_graph(True)
    Fa = t.compute_field_fmm(precision="mixed").cpu().numpy()
    Fa2 = t.compute_field_fmm(precision="mixed").cpu().numpy()  # replayed
    assert np.array_equal(Fa, Fa2)
    t.rebuild(pb)
    Fb = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.times()
    fresh = fg.build_tree(pb, S, pb.shape[0], 128, 8, 0.5)
    fresh.set_tune(impl=3)
    assert np.array_equal(fresh.compute_field_fmm(precision="mixed").cpu().numpy(), Fb)
