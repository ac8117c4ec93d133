"""A demagnetising-field operator in the shape of fidimag's atomistic
`DemagFMM(order, ncrit, theta)`, the external consumer of fmmgen that
fidimag_tests/test_fmm.py:31 times against FFT demag.

Each lattice site i carries a magnetic moment mu_s[i] * m_i (|m_i| = 1).  The
dipolar field at site i, in tesla, is

    B_i = mu0/(4 pi) sum_{j != i} mu_s[j] (3 (m_j . u) u - m_j) / r^3,
    r = |x_i - x_j| unit_length, u = (x_i - x_j)/|x_i - x_j|,

which is minus the field of the FMM's dipole sources (source_order 1, the
potential -s.d/|d|^3 of fmmgen's dipole P2P, example/operators.cpp:54-66,
differentiated exactly).  The site positions are fixed, so the tree and its
interaction lists are built once in `setup`; every `compute_field` uploads the
current spins as dipole sources and runs the device FMM pass.

fidimag keeps vectors flat, [m_x0, m_y0, m_z0, m_x1, ...]; so does this class.
The moments are divided by max(mu_s) before they reach the device and the
field is multiplied back, so the mixed-precision passes see values of order
one rather than ~1e-23 A m^2.
"""
import math

import numpy as np
import torch

from .tree import build_tree

MU0 = 4e-7 * math.pi  # vacuum permeability (fidimag's value, in T m / A)


class DemagFMM:
    """Atomistic demag field by the device FMM.

    order, ncrit, theta: the FMM's expansion order, leaf size and opening angle,
    as fidimag.atomistic.DemagFMM(order, ncrit, theta) takes them.
    precision: "fp64" (default), "mixed" or "mixed_simt", as Tree.compute_field_fmm.
    """

    def __init__(self, order, ncrit, theta, name="DemagFMM", precision="fp64"):
        self.order, self.ncrit, self.theta = int(order), int(ncrit), float(theta)
        self.name = name
        self.precision = precision
        self.jac = False
        self.tree = None

    def setup(self, mesh, spin, mu_s, mu_s_inv=None, unit_length=None):
        """mesh: an object with `coordinates` ([n][3] site positions in units of
        `unit_length`) and `unit_length` (metres), or the [n][3] array itself.
        spin: flat [3n] unit vectors; mu_s: [n] moment magnitudes (A m^2)."""
        coords = getattr(mesh, "coordinates", mesh)
        self.unit_length = float(unit_length if unit_length is not None else getattr(mesh, "unit_length", 1.0))
        pos = np.ascontiguousarray(coords, dtype=np.float64).reshape(-1, 3)
        self.n = pos.shape[0]
        self.spin = spin
        mu = np.broadcast_to(np.asarray(mu_s, dtype=np.float64), (self.n,))
        self.mu_scale = float(np.max(np.abs(mu))) if self.n else 1.0
        if self.mu_scale == 0.0:
            self.mu_scale = 1.0
        self.mu = torch.tensor(mu / self.mu_scale, dtype=torch.float64, device="cuda").reshape(-1, 1)
        self.tree = build_tree(pos, np.zeros((self.n, 3)), self.n, self.ncrit, self.order, self.theta,
                               source_order=1)
        self.coef = -MU0 / (4.0 * math.pi) * self.mu_scale / self.unit_length ** 3
        self.field = np.zeros(3 * self.n)

    def compute_field_device(self, spin):
        """The field as a [n][3] device tensor (tesla) for flat spins `spin`
        (host array or device tensor)."""
        if self.tree is None:
            raise RuntimeError("setup() has not been called")
        m = torch.as_tensor(spin, dtype=torch.float64).to("cuda").reshape(-1, 3)
        if m.shape[0] != self.n:
            raise ValueError(f"expected {3 * self.n} spin components, got {m.numel()}")
        F = self.tree.compute_field_fmm(S=(m * self.mu).contiguous(), potential=False, field=True,
                                        precision=self.precision)
        return F.mul_(self.coef)

    def compute_field(self, t=0, spin=None):
        """fidimag's Energy.compute_field: the flat [3n] field for `spin`
        (default: the spins given to setup)."""
        s = self.spin if spin is None else spin
        self.field = self.compute_field_device(s).cpu().numpy().reshape(-1)
        return self.field

    def compute_energy(self, spin=None):
        """E = -1/2 sum_i mu_s[i] m_i . B_i (joules)."""
        s = self.spin if spin is None else spin
        B = self.compute_field_device(s)
        m = torch.as_tensor(s, dtype=torch.float64).to("cuda").reshape(-1, 3)
        return float(-0.5 * self.mu_scale * (self.mu * m * B).sum())
