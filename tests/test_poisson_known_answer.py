"""Known answer of the Poisson solve on the CPU: the oracle's potential
(the reference's integrated-Green's-function convolution, sc.py:109-168) and
its forward-difference fields (sc.py:195-200) against the closed-form
potential and field of a Gaussian bunch.

The reference's own tests check particles only against earlier runs of the
same code; this checks the method against physics.  The charge grid is the
midpoint rule of the Gaussian density on the nodes, so the errors are the
discretisation's, O(h^2): measured 7.6e-4 (phi) and 4.8e-3 (E) on 32^3 at
h = 0.26 sigma, 2.3e-4 and 1.2e-3 on 64^3 at h = 0.13 sigma.  The bounds
below sit about 30% above those figures, and refining the mesh must cut the
potential's error at least threefold.
"""
import numpy as np
import pytest
from scipy.special import erf

import gauss_field as G
from oracle import sc_oracle

Q = 1e-9


def test_closed_form_matches_the_round_bunch_potential():
    """The quadrature against the erf form of a spherical Gaussian."""
    s = 1e-3
    rng = np.random.default_rng(3)
    pts = rng.normal(size=(200, 3)) * 2 * s
    phi, E = G.potential_and_field(pts, (s, s, s), Q)
    r = np.linalg.norm(pts, axis=1)
    phi_ex = G.COULOMB * Q * erf(r / (np.sqrt(2) * s)) / r
    er = G.COULOMB * Q * (erf(r / (np.sqrt(2) * s)) / r ** 2
                          - np.sqrt(2 / np.pi) / s * np.exp(-r ** 2 / (2 * s * s)) / r)
    assert np.abs(phi - phi_ex).max() <= 1e-9 * np.abs(phi_ex).max()
    assert np.abs(E - er[:, None] * pts / r[:, None]).max() <= 1e-9 * np.abs(er).max()


@pytest.mark.parametrize("nmesh,sigma,bound_phi,bound_e", [
    ((32, 32, 32), (1e-3, 1e-3, 1e-3), 1.0e-3, 6.5e-3),
    # the rest-frame shape of the 130 MeV benchmark bunch: cells 500x longer than wide
    ((32, 32, 64), (50e-6, 50e-6, 25e-3), 4.2e-4, 4.3e-3),
])
def test_oracle_potential_and_field_against_closed_form(nmesh, sigma, bound_phi, bound_e):
    pos, h, q = G.node_grid(nmesh, sigma, Q)
    phi = sc_oracle.potential(q, h)
    e_phi, e_field = G.grid_errors(phi, pos, h, sigma, Q)
    assert e_phi <= bound_phi, e_phi
    assert max(e_field) <= bound_e, e_field


def test_oracle_potential_converges_at_second_order():
    sigma = (1e-3, 1e-3, 1e-3)
    errs = []
    for n in (16, 32):
        pos, h, q = G.node_grid((n, n, n), sigma, Q)
        errs.append(G.grid_errors(sc_oracle.potential(q, h), pos, h, sigma, Q)[0])
    assert errs[1] <= errs[0] / 3, errs
