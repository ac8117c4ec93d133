"""The generated M2L kernels' plan (fmmgen_gb300/gen_m2l_cm.py), checked on the
CPU: every family's kernels together issue each term of the order-pmax M2L
exactly once, with the right derivative index; each output group is stored by
its first kernel and added to by the others; kernel bodies stay within the
code bound; the degree nest makes truncation at any order q <= pmax keep
exactly the terms |n| + |m| <= q; and the generated sources on disk are the
generator's current output."""
import os

import numpy as np
import pytest

from fmmgen_gb300 import gen_m2l_cm as g


def mono(p):
    return g.monomials(p)


@pytest.mark.parametrize("so,pmax", g.FAMILIES)
def test_terms_cover_the_translation_once(so, pmax):
    m_ = mono(pmax)
    moff = g.nterms(so - 1)
    want = set()
    for i in range(g.nterms(pmax - so)):
        for j in range(moff, g.nterms(pmax)):
            n, m = m_[i], m_[j]
            if sum(m) >= so and sum(n) + sum(m) <= pmax:
                want.add((i, j - moff))
    got = []
    for kern in g.plan(so, pmax):
        outs = set(kern["outs"])
        for c in kern["chunks"]:
            for d, k, i, jj in c["terms"]:
                assert i in outs and c["mb"] <= jj < c["me"]
                n, m = m_[i], m_[jj + moff]
                assert d == sum(n) + sum(m)
                assert k == g.idx3((n[0] + m[0], n[1] + m[1], n[2] + m[2]))
                got.append((i, jj))
    assert len(got) == len(set(got)) and set(got) == want


@pytest.mark.parametrize("so,pmax", g.FAMILIES)
def test_groups_store_once_and_bound_code(so, pmax):
    kernels = g.plan(so, pmax)
    firsts = {}
    covered = []
    for kern in kernels:
        key = tuple(kern["outs"])
        if kern["first"]:
            assert key not in firsts
            firsts[key] = True
            covered += kern["outs"]
        else:
            assert key in firsts  # a later kernel of a group adds to what its first stored
        nf = sum(len(c["terms"]) for c in kern["chunks"])
        assert nf <= g.KERNEL_FMAS or len(kern["chunks"]) == 1
        # chunks of a kernel are consecutive and start on float4 boundaries
        for a, b in zip(kern["chunks"], kern["chunks"][1:]):
            assert a["me"] == b["mb"]
        assert all(c["mb"] % 4 == 0 for c in kern["chunks"])
    assert sorted(covered) == list(range(g.nterms(pmax - so)))


@pytest.mark.parametrize("so,pmax", [(0, 12), (1, 8)])
def test_truncation_by_degree_of_k(so, pmax):
    """A lane at order q runs exactly the terms of degree <= q (the nest),
    and the kernels a pass of order p launches hold all terms of degree <= p."""
    m_ = mono(pmax)
    moff = g.nterms(so - 1)
    for q in range(so + 1, pmax + 1):
        kept = set()
        for kern in g.plan(so, pmax):
            if g.kernel_dmin(kern) > q:
                continue  # not launched at order q
            for c in kern["chunks"]:
                if kern["lo"] + c["emin"] > q:
                    continue  # chunk skipped by the warp-uniform count
                kept |= {(i, jj) for d, k, i, jj in c["terms"] if d <= q}
        want = {(i, j - moff) for i in range(g.nterms(q - so)) for j in range(moff, g.nterms(q))
                if sum(m_[j]) >= so and sum(m_[i]) + sum(m_[j]) <= q}
        assert kept == want, q


def test_generated_sources_are_current(tmp_path, monkeypatch):
    monkeypatch.setattr(g, "CSRC", str(tmp_path))
    g.generate()
    for so, pmax in g.FAMILIES:
        fn = g.family_file(so, pmax)
        with open(os.path.join(tmp_path, fn)) as a, open(os.path.join(os.path.dirname(g.__file__), "csrc", fn)) as b:
            assert a.read() == b.read(), fn
    with open(os.path.join(tmp_path, "m2l_cm.cuh")) as a, \
            open(os.path.join(os.path.dirname(g.__file__), "csrc", "m2l_cm.cuh")) as b:
        assert a.read() == b.read()


def test_numeric_contraction_matches_direct():
    """The plan's terms, evaluated in numpy with the kernels' grouping (per-pair
    sums for the outputs marked), equal the direct contraction."""
    so, pmax = 0, 8
    m_ = mono(pmax)
    rng = np.random.default_rng(3)
    D = rng.standard_normal(g.nterms(pmax))
    M = rng.standard_normal(g.nterms(pmax))
    ref = np.zeros(g.nterms(pmax))
    for i in range(g.nterms(pmax)):
        for j in range(g.nterms(pmax)):
            n, m = m_[i], m_[j]
            if sum(n) + sum(m) <= pmax:
                ref[i] += D[g.idx3((n[0] + m[0], n[1] + m[1], n[2] + m[2]))] * M[j]
    L = np.zeros_like(ref)
    for kern in g.plan(so, pmax):
        acc = {i: 0.0 for i in kern["outs"]}
        for c in kern["chunks"]:
            for d, k, i, jj in c["terms"]:
                acc[i] += D[k] * M[jj]
        for i, v in acc.items():
            L[i] = v if kern["first"] else L[i] + v
    assert np.allclose(L, ref, rtol=1e-12, atol=1e-12)
