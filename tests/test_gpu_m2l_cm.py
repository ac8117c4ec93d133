"""Generated CUDA-core M2L for every order up to 12 (csrc/m2l_cm_s*.cu), both
schedules: class-major (impl 4: a warp takes 32 target cells' pairs of one
translation class per step) and target-major (impl 5: a thread per target
cell over its list).  Against the FP64 pass and the FP32 contraction engine
(impl 2) on uniform and adaptive trees, every order of both families,
per-pair orders (each lane truncating at its pair's order), determinism and
the empty-list case."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def system(kind, n, so, seed):
    rng = np.random.default_rng(seed)
    if kind == "uniform":
        pos = rng.uniform(0, 1, (n, 3))
    else:  # Plummer sphere: deep, adaptive levels and pairs across levels
        r = 0.1 / np.sqrt(rng.uniform(0.01, 1.0, n) ** (-2.0 / 3.0) - 1.0)
        v = rng.standard_normal((n, 3))
        pos = v / np.linalg.norm(v, axis=1, keepdims=True) * r[:, None]
    S = rng.uniform(-1, 1, (n, 1)) if so == 0 else rng.standard_normal((n, 3))
    return torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda")


@pytest.mark.parametrize("so,p", [(0, 2), (0, 4), (0, 6), (0, 8), (0, 10), (0, 12), (1, 3), (1, 6), (1, 8)])
@pytest.mark.parametrize("kind", ["uniform", "plummer"])
@pytest.mark.parametrize("impl", [4, 5])
def test_fixed_order_vs_fp64_and_engine(fg, impl, kind, so, p):
    pos, S = system(kind, 40000, so, 100 + 10 * p + so)
    t = fg.build_tree(pos, S, pos.shape[0], 64, p, 0.5, source_order=so)
    F64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
    _, L64 = t.expansions()
    t.set_tune(impl=2)
    Fe = t.compute_field_fmm(precision="mixed").cpu().numpy()
    _, Le = t.expansions()
    t.set_tune(impl=impl)
    Fc = t.compute_field_fmm(precision="mixed").cpu().numpy()
    _, Lc = t.expansions()
    assert np.array_equal(Fc, t.compute_field_fmm(precision="mixed").cpu().numpy())  # deterministic
    e_c, e_e = rel(Lc, L64), rel(Le, L64)
    assert e_c < max(2 * e_e, 1e-6), (e_c, e_e)
    fe_c, fe_e = rel(Fc[:, -3:], F64[:, -3:]), rel(Fe[:, -3:], F64[:, -3:])
    assert fe_c < max(2 * fe_e, 5e-7), (fe_c, fe_e)


@pytest.mark.parametrize("so,p", [(0, 12), (0, 8), (1, 6)])
@pytest.mark.parametrize("impl", [4, -1])
def test_per_pair_orders(fg, impl, so, p):
    """Random per-pair orders: the generated kernels against the FP64 pass with
    the same orders, and no worse than the engine's mixed pass."""
    pos, S = system("plummer", 30000, so, 200 + p)
    t = fg.build_tree(pos, S, pos.shape[0], 64, p, 0.5, source_order=so)
    rng = np.random.default_rng(300 + p)
    t.set_m2l_orders(rng.integers(0, p + 2, t.nm2l).astype(np.uint8))
    F64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
    t.set_tune(impl=2)  # per-pair orders on the engine
    Fe = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.set_tune(impl=impl)  # class-major, or the default: target-major
    Fc = t.compute_field_fmm(precision="mixed").cpu().numpy()
    assert np.array_equal(Fc, t.compute_field_fmm(precision="mixed").cpu().numpy())
    fe_c, fe_e = rel(Fc, F64), rel(Fe, F64)
    assert fe_c < max(2 * fe_e, 5e-7), (fe_c, fe_e)
    # the truncation is real: all pairs at order p give another field
    t.set_m2l_orders(None)
    t.set_tune(impl=5)
    Ff = t.compute_field_fmm(precision="mixed").cpu().numpy()
    assert rel(Ff, Fc) > 10 * fe_c


@pytest.mark.parametrize("impl", [4, 5])
def test_uniform_orders_equal_fixed(fg, impl):
    """Every pair at order p through the per-pair path gives the fixed-order
    pass bit for bit (the same kernels, every lane at p)."""
    pos, S = system("uniform", 30000, 0, 7)
    t = fg.build_tree(pos, S, pos.shape[0], 64, 9, 0.5)
    t.set_tune(impl=impl)
    ref = t.compute_field_fmm(precision="mixed").cpu().numpy()
    t.set_m2l_orders(np.full(t.nm2l, 9, np.uint8))
    assert np.array_equal(t.compute_field_fmm(precision="mixed").cpu().numpy(), ref)


@pytest.mark.parametrize("impl", [4, 5])
def test_no_pairs(fg, impl):
    pos, S = system("uniform", 50, 0, 8)
    t = fg.build_tree(pos, S, 50, 64, 8, 0.5)
    assert t.nm2l == 0
    t.set_tune(impl=impl)
    F = t.compute_field_fmm(precision="mixed").cpu().numpy()
    F64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
    assert rel(F, F64) < 1e-6


@pytest.mark.parametrize("impl", [3, 0, 1, 2, 4, 5])
def test_kernel_times(fg, impl):
    """Every M2L implementation brackets its kernels with events: the kernel
    time is positive and within the M2L phase of the pass."""
    pos, S = system("uniform", 40000, 0, 9)
    t = fg.build_tree(pos, S, pos.shape[0], 64, 6, 0.5)
    t.set_tune(impl=impl)
    t.compute_field_fmm(precision="mixed")
    k = t.kernel_ms()
    ph = t.times()[1]
    assert k["M2L"] > 0 and k["P2P"] > 0, k
    assert k["M2L"] <= ph["M2L"] + 1e-3, (k, ph)
