"""The fidimag-style demag operator (fmmgen_gb300.demag.DemagFMM, the consumer
of fidimag_tests/test_fmm.py:31).  fidimag itself is not installed: the field
is checked against the dipolar sum written out in numpy, and against the CPU
restatement's FMM on the same tree."""
import math

import numpy as np
import pytest

MU_B = 9.274009994e-24
MU0 = 4e-7 * math.pi


def lattice(L, a=0.2715, seed=5):
    g = np.arange(L) * a
    pos = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    rng = np.random.default_rng(seed)
    m = rng.standard_normal((len(pos), 3))
    m /= np.linalg.norm(m, axis=1, keepdims=True)
    return pos, m


def dipolar_field(pos, m, mu, unit_length):
    """B_i = mu0/(4 pi) sum_{j != i} mu_j (3 (m_j.u) u - m_j) / r^3, in tesla."""
    d = pos[:, None, :] - pos[None, :, :]
    r = np.linalg.norm(d, axis=-1)
    np.fill_diagonal(r, np.inf)
    u = d / r[..., None]
    mu_ = np.broadcast_to(mu, (len(pos),))
    mdotu = np.einsum("jk,ijk->ij", m, u)
    B = (mu_[None, :, None] * (3 * mdotu[..., None] * u - m[None, :, :]) / (r ** 3)[..., None]).sum(1)
    return MU0 / (4 * math.pi) * B / unit_length ** 3


def test_dipole_sources_are_minus_the_dipolar_field(oracle_lib):
    """The identity DemagFMM rests on: the field of fmmgen's dipole sources
    (evaluate_direct, example/calculate.cpp:252-264) is minus the magnetic
    dipolar kernel (3(m.u)u - m)/r^3."""
    pos, m = lattice(6)
    F = oracle_lib.direct(pos, m, source_order=1, potential=False)
    B = dipolar_field(pos, m, 1.0, 1.0) * (4 * math.pi) / MU0
    assert np.abs(-F - B).max() <= 1e-13 * np.abs(B).max()


def test_compute_before_setup_raises():
    from fmmgen_gb300.demag import DemagFMM

    with pytest.raises(RuntimeError):
        DemagFMM(8, 32, 0.5).compute_field_device(np.zeros(3))


class _Mesh:
    def __init__(self, coords, unit_length):
        self.coordinates = coords
        self.unit_length = unit_length


@pytest.mark.gpu
def test_demag_field_vs_dipolar_sum_and_checker(fg, oracle_lib):
    from fmmgen_gb300.demag import DemagFMM

    pos, m = lattice(12)
    mu = 3 * MU_B
    dm = DemagFMM(8, 32, 0.5)
    dm.setup(_Mesh(pos, 1e-9), m.reshape(-1), np.full(len(pos), mu))
    B = dm.compute_field().reshape(-1, 3)
    Bx = dipolar_field(pos, m, mu, 1e-9)
    assert np.linalg.norm(B - Bx) / np.linalg.norm(Bx) < 1e-4
    # the same FMM on the CPU (same tree, order, theta)
    t = oracle_lib.OracleTree(pos, m, 32, 8, 0.5, 1)
    Fo, _ = t.evaluate(potential=False)
    Bo = -MU0 / (4 * math.pi) * mu / 1e-27 * Fo
    assert np.linalg.norm(B - Bo) / np.linalg.norm(Bo) < 1e-10
    # energy, -1/2 sum mu m.B
    assert abs(dm.compute_energy() - (-0.5 * mu * np.sum(m * Bx))) <= 1e-4 * abs(0.5 * mu * np.sum(m * Bx)) + 1e-30


@pytest.mark.gpu
def test_demag_new_spins_and_precision(fg):
    from fmmgen_gb300.demag import DemagFMM

    pos, m = lattice(10, seed=1)
    _, m2 = lattice(10, seed=2)
    mu = np.random.default_rng(3).uniform(1.0, 3.0, len(pos)) * MU_B
    dm = DemagFMM(10, 16, 0.4)
    dm.setup(pos, m.reshape(-1), mu, unit_length=1e-9)
    B1 = dm.compute_field().copy()
    B2 = dm.compute_field(spin=m2.reshape(-1)).copy()
    for spin, B in ((m, B1), (m2, B2)):
        Bx = dipolar_field(pos, spin, mu, 1e-9).reshape(-1)
        assert np.linalg.norm(B - Bx) / np.linalg.norm(Bx) < 5e-6
    mixed = DemagFMM(10, 16, 0.4, precision="mixed")
    mixed.setup(pos, m2.reshape(-1), mu, unit_length=1e-9)
    Bm = mixed.compute_field()
    assert np.linalg.norm(Bm - B2) / np.linalg.norm(B2) < 1e-5
