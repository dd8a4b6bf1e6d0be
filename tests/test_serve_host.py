"""Requests the tracking server refuses at submit (host checks, no GPU): a
beam whose charge array does not match its particles, an energy at or below
the electron's rest energy, a malformed particle array or mesh, and a line
without tracking steps.  A job that passed these checks is batched with the
others, so none of them may be left to a later tick."""
import numpy as np
import pytest

from ocelot_gb300 import ParticleArray
from ocelot_gb300 import serve as S
from ocelot_gb300.globals import m_e_GeV


def _pa(n, E=0.13, nq=None):
    pa = ParticleArray(n)
    pa.rparticles[:] = np.random.default_rng(1).standard_normal((6, n)) * 1e-4
    pa.q_array = np.full(n if nq is None else nq, 1e-12)
    pa.E = E
    return pa


def test_a_valid_request_gives_its_steps():
    steps = S.validate_request(S.Request(_pa(100), S.fodo(1), (15, 15, 15), 0.25, 1))
    assert len(steps) == 10       # 2.4 m of FODO cell in steps of 0.25 m
    assert len(S.validate_request(S.Request(S.BeamSpec(n=10, seed=1), S.fodo(1), (8, 8, 8)))) == 10


@pytest.mark.parametrize("nq", [99, 101, 0])
def test_charge_array_of_another_length_is_refused(nq):
    with pytest.raises(ValueError, match="q_array has"):
        S.validate_request(S.Request(_pa(100, nq=nq), S.fodo(1), (15, 15, 15)))


@pytest.mark.parametrize("E", [0.0, -0.1, m_e_GeV, 0.5 * m_e_GeV, float("nan"), float("inf")])
def test_energy_at_or_below_the_rest_energy_is_refused(E):
    with pytest.raises(ValueError, match="rest energy"):
        S.validate_request(S.Request(_pa(100, E=E), S.fodo(1), (15, 15, 15)))
    with pytest.raises(ValueError, match="rest energy"):
        S.validate_request(S.Request(S.BeamSpec(n=100, seed=1, energy_gev=E), S.fodo(1), (15, 15, 15)))


def test_malformed_beams_and_meshes_are_refused():
    pa = _pa(100)
    pa.rparticles = np.zeros((5, 100))
    with pytest.raises(ValueError, match="shape"):
        S.validate_request(S.Request(pa, S.fodo(1), (15, 15, 15)))
    with pytest.raises(ValueError, match="at least one particle"):
        S.validate_request(S.Request(S.BeamSpec(n=0, seed=1), S.fodo(1), (15, 15, 15)))
    for mesh in [(15, 15), (3, 15, 15)]:
        with pytest.raises(ValueError, match="nmesh"):
            S.validate_request(S.Request(_pa(100), S.fodo(1), mesh))


def test_line_without_steps_is_refused():
    with pytest.raises(ValueError, match="no tracking steps"):
        S.validate_request(S.Request(_pa(100), S.fodo(0), (15, 15, 15)))
