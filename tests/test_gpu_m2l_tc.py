"""Tensor-core M2L (tcgen05 kind::f16, 3 FP16 products per term) of the mixed pass against the FP64 pass
and the FP32 CUDA-core M2L kernels, on the local expansions every cell ends
with and on the field."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def plummer(rng, n):
    r = 1.0 / np.sqrt(rng.uniform(0.01, 1.0, n) ** (-2.0 / 3.0) - 1.0)
    v = rng.standard_normal((n, 3))
    return v / np.linalg.norm(v, axis=1, keepdims=True) * r[:, None]


def system(dist, so, n, seed):
    rng = np.random.default_rng(seed)
    if dist == "uniform":
        pos = rng.uniform(0, 1, (n, 3))
    elif dist == "plummer":
        pos = plummer(rng, n)
    else:  # a few dense clusters in an empty box
        c = rng.uniform(0, 1, (8, 3))
        pos = c[rng.integers(0, 8, n)] + 0.01 * rng.standard_normal((n, 3))
    S = rng.uniform(-1, 1, (n, 1)) if so == 0 else rng.standard_normal((n, 3))
    return torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda")


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


CASES = [(8, 0, "uniform", 64), (9, 0, "uniform", 64), (6, 1, "plummer", 32), (7, 1, "uniform", 64),
         (4, 0, "clustered", 16), (2, 0, "uniform", 8), (5, 1, "clustered", 24)]


@pytest.mark.parametrize("p,so,dist,ncrit", CASES)
def test_tc_m2l_local_expansions(fg, p, so, dist, ncrit):
    pos, S = system(dist, so, 30000, 100 + p)
    t = fg.build_tree(pos, S, pos.shape[0], ncrit, p, 0.5, source_order=so)
    F64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
    _, L64 = t.expansions()
    Ftc = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.times()  # raises if a pipeline wait of the tensor-core kernel timed out
    _, Ltc = t.expansions()
    # the pipeline is deterministic: a second pass gives the same bits
    Ftc2 = t.compute_field_fmm(precision="mixed").cpu().numpy()
    assert np.array_equal(Ftc, Ftc2)
    Fs = t.compute_field_fmm(precision="mixed_simt").cpu().numpy()
    _, Ls = t.expansions()
    # the 3xFP16 products carry ~2^-22 relative error against FP32's 2^-24:
    # the local expansions stay within a few times the CUDA-core FP32 error
    e_tc, e_s = rel(Ltc, L64), rel(Ls, L64)
    assert e_tc < max(8 * e_s, 1e-6), (e_tc, e_s)
    # and the field within the mixed tolerance of the FP64 pass
    assert rel(Ftc[:, -3:], F64[:, -3:]) < 2e-6
    assert rel(Ftc[:, 0], F64[:, 0]) < 2e-6


def test_tc_m2l_rebuild_refreshes_operators(fg):
    """The per-class operator records follow a rebuild with new classes."""
    pos, S = system("uniform", 0, 20000, 7)
    t = fg.build_tree(pos, S, pos.shape[0], 64, 8, 0.5)
    t.compute_field_fmm(precision="mixed")
    pos2, _ = system("plummer", 0, 20000, 8)
    t.rebuild(pos2)
    Ftc = t.compute_field_fmm(precision="mixed").cpu().numpy()
    F64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
    t.times()
    assert rel(Ftc[:, -3:], F64[:, -3:]) < 2e-6


def test_tc_m2l_rebuild_same_classes(fg):
    """A rebuild whose translation classes equal the previous build's reuses the
    per-class operator data; results match a fresh tree bit for bit, also when
    position sets alternate (A, B, A)."""
    pa, S = system("uniform", 0, 20000, 11)
    pb, _ = system("clustered", 0, 20000, 12)
    t = fg.build_tree(pa, S, pa.shape[0], 64, 8, 0.5)
    Fa = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.rebuild(pa)
    assert np.array_equal(t.compute_field_fmm(precision="mixed").cpu().numpy(), Fa)
    t.rebuild(pb)
    Fb = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.rebuild(pa)
    assert np.array_equal(t.compute_field_fmm(precision="mixed").cpu().numpy(), Fa)
    fresh = fg.build_tree(pb, S, pb.shape[0], 64, 8, 0.5)
    assert np.array_equal(fresh.compute_field_fmm(precision="mixed").cpu().numpy(), Fb)
    t.times()
