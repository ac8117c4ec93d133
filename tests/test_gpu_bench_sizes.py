"""Parity at the benchmarked sizes: the device tree and interaction lists of
bench.py's workloads are bit-exact against the CPU restatement of build_tree /
interact_dehnen_lazy (example/tree.cpp:130-233, example/calculate.cpp:81-133),
and the headline's mixed and FP64 fields match the restatement's FP64
compute_field_fmm on a subset of target cells.

Workloads (the inputs bench.py generates, same seeds):
  * 10^6 charges uniform in the unit cube, ncrit 128, theta 0.5, p 8 (headline);
  * 2x10^6 dipoles in a Plummer sphere (scale 0.1, truncated at 1), ncrit 64,
    theta 0.5, p 6."""
import hashlib
import types

import numpy as np
import pytest
import torch

from test_gpu_tree import canonical, check_against

pytestmark = pytest.mark.gpu


def bench_inputs(dist, n, so, seed=0):
    import bench

    a = types.SimpleNamespace(dist=dist, n=n, so=so)
    return bench.workload(a, seed)


def oracle_vs_device(fg, oracle_lib, pos, S, ncrit, p, theta, so):
    ot = oracle_lib.OracleTree(pos, S, ncrit, p, theta, so)
    oc = ot.cells()
    o = np.argsort(oc["id"])
    om, op = ot.lists()
    dm = hashlib.sha256(canonical(om).tobytes()).hexdigest()
    dp = hashlib.sha256(canonical(op).tobytes()).hexdigest()
    nm, npp = len(om), len(op)
    del om, op
    t = fg.build_tree(torch.tensor(pos, device="cuda"), torch.tensor(S, device="cuda"), len(pos), ncrit, p, theta,
                      source_order=so)
    check_against(t, oc["id"][o], oc["nleaf"][o], oc["centre"][o], oc["id"][oc["leaf_cell"]], oc["leaf_off"],
                  oc["leaf_idx"], dm, dp, nm, npp)
    return t, ot


def test_headline_tree_and_fields_vs_oracle(fg, oracle_lib):
    pos, S = bench_inputs("uniform", 1_000_000, 0)
    t, ot = oracle_vs_device(fg, oracle_lib, pos, S, 128, 8, 0.5, 0)
    assert (t.ncells, t.nm2l) == (37449, 15678688)
    # the restatement's exact FP64 FMM at the particles of every 97th leaf (about 10^4 targets)
    Fo, _ = ot.evaluate(potential=False, field=True, sample_stride=-97)
    rows = np.flatnonzero(np.any(Fo != 0.0, axis=1))
    assert 5_000 < len(rows) < 20_000
    Fm = t.compute_field_fmm(potential=False, field=True, precision="mixed").cpu().numpy()
    F64 = t.compute_field_fmm(potential=False, field=True, precision="fp64").cpu().numpy()
    ref = Fo[rows]
    e64 = np.linalg.norm(F64[rows] - ref) / np.linalg.norm(ref)
    emx = np.linalg.norm(Fm[rows] - ref) / np.linalg.norm(ref)
    assert e64 < 1e-10, e64
    # the mixed pass differs from the FP64 FMM by its rounding only (the FP64
    # FMM's own truncation error here is 2.4e-6)
    assert emx < 5e-7, emx


def test_plummer_dipole_tree_vs_oracle(fg, oracle_lib):
    pos, S = bench_inputs("plummer", 2_000_000, 1)
    t, _ = oracle_vs_device(fg, oracle_lib, pos, S, 64, 6, 0.5, 1)
    assert t.nm2l > 10_000_000
