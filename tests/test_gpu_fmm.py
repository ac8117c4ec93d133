"""Whole-FMM parity: the device evaluation pass against the reference's
compute_field_fmm (golden F), the CPU restatement, and the FP64 direct sum."""
import os

import numpy as np
import pytest
import torch

from conftest import GOLDEN

pytestmark = pytest.mark.gpu
TREES = ["uniform10k", "deep", "dipole_plummer", "clustered", "tiny", "example_scaled"]

# FP64 path vs the reference's FP64 FMM: same algorithm, different summation
# order, and M2L operators built from the ideal (exactly scaled) displacement of
# each translation class instead of the FP64 centre difference.
TOL_FP64 = 1e-10
# Mixed path: FP32 arithmetic everywhere except operator assembly and the final
# accumulation; it must stay far below the p=8 truncation error (~2e-6).
TOL_MIXED = 2e-6


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


def run(fg, g, precision="fp64"):
    pos = torch.tensor(g["pos"], device="cuda")
    S = torch.tensor(g["S"], device="cuda")
    t = fg.build_tree(pos, S, int(g["N"]), int(g["ncrit"]), int(g["order"]), float(g["theta"]),
                      source_order=int(g["source_order"]))
    return t, t.compute_field_fmm(precision=precision).cpu().numpy()


@pytest.mark.parametrize("case", TREES)
def test_fp64_fmm_vs_reference(fg, case):
    g = np.load(os.path.join(GOLDEN, f"tree_{case}.npz"))
    _, F = run(fg, g)
    assert rel(F, g["F"]) < TOL_FP64


@pytest.mark.parametrize("case", TREES)
def test_mixed_fmm_vs_reference(fg, case):
    g = np.load(os.path.join(GOLDEN, f"tree_{case}.npz"))
    _, F = run(fg, g, "mixed")
    assert rel(F[:, 1:], g["F"][:, 1:]) < TOL_MIXED
    assert rel(F[:, 0], g["F"][:, 0]) < TOL_MIXED


def test_expansions_match_checker(fg, oracle_lib):
    """Per-cell M and L (unscaled back to fmmgen's convention) vs the restatement."""
    g = np.load(os.path.join(GOLDEN, "tree_uniform10k.npz"))
    t, _ = run(fg, g)
    M, L = t.expansions()
    ot = oracle_lib.OracleTree(g["pos"], g["S"], 64, 4, 0.5, 0)
    _, _, Mo, Lo = ot.evaluate(want_ML=True)
    oc = ot.cells()
    gc = t.cells()
    om = {int(i): k for k, i in enumerate(oc["id"])}
    perm = np.array([om[int(i)] for i in gc["id"]])
    for a, b in ((M, Mo[perm]), (L, Lo[perm])):
        err = np.max(np.abs(a - b), axis=1) / np.maximum(np.max(np.abs(b), axis=1), 1e-300)
        assert err.max() < 1e-10


@pytest.mark.parametrize("so,p", [(0, 8), (1, 6), (0, 12)])
def test_fmm_vs_direct(fg, so, p):
    rng = np.random.default_rng(40 + p)
    N = 20000
    pos = rng.uniform(0, 1, (N, 3))
    S = rng.uniform(-1, 1, (N, 1)) if so == 0 else rng.standard_normal((N, 3))
    pos_t, S_t = torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda")
    t = fg.build_tree(pos_t, S_t, N, 64, p, 0.5, source_order=so)
    F64 = t.compute_field_fmm(precision="fp64").cpu().numpy()
    F32 = t.compute_field_fmm(precision="mixed").cpu().numpy()
    tg = np.arange(0, N, 5)
    Fd = fg.direct(pos_t, S_t, targets=tg, source_order=so).cpu().numpy()
    e64 = rel(F64[tg, 1:], Fd[:, 1:])
    e32 = rel(F32[tg, 1:], Fd[:, 1:])
    bound = {8: 1e-5, 6: 1e-5, 12: 1e-7}[p]
    assert e64 < bound
    # mixed precision adds at most ~10% on top of the truncation error at p <= 8
    assert e32 < max(1.1 * e64, 5e-7)


def test_direct_vs_checker(fg, oracle_lib):
    rng = np.random.default_rng(2)
    for so in (0, 1):
        N = 3000
        pos = rng.uniform(-1, 1, (N, 3))
        S = rng.standard_normal((N, 1 if so == 0 else 3))
        tg = np.arange(0, N, 3)
        Fg = fg.direct(torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda"), targets=tg,
                       source_order=so).cpu().numpy()
        Fo = oracle_lib.direct(pos, S, tg, so)
        assert rel(Fg, Fo) < 1e-13


def test_output_switches(fg):
    g = np.load(os.path.join(GOLDEN, "tree_deep.npz"))
    t, F = run(fg, g)
    pot = t.compute_field_fmm(potential=True, field=False).cpu().numpy()
    fld = t.compute_field_fmm(potential=False, field=True).cpu().numpy()
    assert pot.shape == (3000, 1) and fld.shape == (3000, 3)
    assert np.array_equal(pot[:, 0], F[:, 0]) and np.array_equal(fld, F[:, 1:])


def test_host_arrays_roundtrip(fg):
    """numpy in, numpy out (copies inside the call), same result as device tensors."""
    g = np.load(os.path.join(GOLDEN, "tree_deep.npz"))
    t = fg.build_tree(g["pos"], g["S"], 3000, 8, 3, 0.7)
    F = np.zeros((3000, 4))
    t.compute_field_fmm(F)
    _, Fd = run(fg, g)
    assert np.array_equal(F, Fd)


def test_monopole_conservation_large(fg):
    """M_sanity_check (example/calculate.cpp:9-21) at 1M: root M0 = sum of charges,
    and mixed vs FP64 agree on a 1M-particle system."""
    rng = np.random.default_rng(77)
    N = 1_000_000
    pos = torch.tensor(rng.uniform(0, 1, (N, 3)), device="cuda")
    q = torch.tensor(rng.uniform(-1, 1, (N, 1)), device="cuda")
    t = fg.build_tree(pos, q, N, 128, 4, 0.5)
    F64 = t.compute_field_fmm(precision="fp64")
    M, _ = t.expansions()
    assert abs(M[0, 0] - q.sum().item()) < 1e-9 * q.abs().sum().item()
    F32 = t.compute_field_fmm(precision="mixed")
    e = (torch.linalg.norm(F32[:, 1:] - F64[:, 1:]) / torch.linalg.norm(F64[:, 1:])).item()
    assert e < 1e-6
