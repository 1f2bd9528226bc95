"""Transition dipoles on the GPU (bse_transition_dipoles) against the restated
Orbitals::CalcCoupledTransition_Dipoles (oracle/orbitals_oracle.py) and the reference's
osc_strength known answers (test_orbitals.cc:202-256): restricted TDA singlets of the golden
methane case, full-BSE states (X + Y), and combined UKS excitons (both spin blocks)."""
import os

import numpy as np
import pytest

from oracle import gaussian_integrals as gi
from oracle.orbitals_oracle import oscillator_strengths, transition_dipoles as oracle_td
from tests.conftest import is_approx

pytestmark = pytest.mark.gpu

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_golden_methane_oscillator_strengths():
    from votca_gb300.bse import oscillator_strengths as osc_gpu
    from votca_gb300.bse import transition_dipoles

    g = np.load(os.path.join(GOLD, "orbitals_osc.npz"))
    basis = gi.parse_basis(str(g["basis_xml"]))
    shells = gi.build_shells([(str(e), tuple(x)) for e, x in zip(g["elements"], g["xyz"])], basis)
    D = gi.dipole(shells)
    td = transition_dipoles(D, g["MOs"], homo=3, vmin=0, cmax=16, X=g["spsi"])
    ref = oracle_td(D, g["MOs"], 0, 4, 4, 13, g["spsi"])
    assert np.abs(td - ref).max() <= 1e-13 * np.abs(ref).max()
    for s in range(3):
        assert is_approx(td[s], g["dipoles_ref"][s], 1e-4)
    osc = osc_gpu(g["omega"], td)
    assert is_approx(osc, g["oscs_ref"], 1e-4)
    assert np.allclose(osc, oscillator_strengths(g["omega"], ref), rtol=1e-12)


def test_full_bse_states_and_offsets():
    """X + Y, a BSE window not starting at level 0, more AO functions than MOs used."""
    from votca_gb300.bse import transition_dipoles

    rng = np.random.default_rng(5)
    nbf, nmo, vmin, homo, cmax, ns = 23, 21, 2, 7, 18, 5
    A = rng.standard_normal((3, nbf, nbf))
    A = A + A.transpose(0, 2, 1)
    C = rng.standard_normal((nbf, nmo))
    vt, ct = homo - vmin + 1, cmax - homo
    X, Y = rng.standard_normal((vt * ct, ns)), 0.1 * rng.standard_normal((vt * ct, ns))
    td = transition_dipoles(A, C, homo, vmin, cmax, X, Y)
    ref = oracle_td(A, C, vmin, vt, homo + 1, ct, X, Y)
    assert np.abs(td - ref).max() <= 1e-12 * np.abs(ref).max()


def test_uks_excitons():
    from votca_gb300.bse import transition_dipoles_uks

    rng = np.random.default_rng(6)
    nbf, vmin, ha, hb, cmax, ns = 17, 0, 4, 3, 14, 4
    A = rng.standard_normal((3, nbf, nbf))
    A = A + A.transpose(0, 2, 1)
    Ca, Cb = rng.standard_normal((nbf, nbf)), rng.standard_normal((nbf, nbf))
    na, nb = (ha - vmin + 1) * (cmax - ha), (hb - vmin + 1) * (cmax - hb)
    X = rng.standard_normal((na + nb, ns))
    td = transition_dipoles_uks(A, Ca, Cb, ha, hb, vmin, cmax, X)
    ref = (oracle_td(A, Ca, vmin, ha - vmin + 1, ha + 1, cmax - ha, X[:na], prefactor=-1.0)
           + oracle_td(A, Cb, vmin, hb - vmin + 1, hb + 1, cmax - hb, X[na:], prefactor=-1.0))
    assert np.abs(td - ref).max() <= 1e-12 * np.abs(ref).max()
    # a beta channel without occupied levels in the window: the alpha block alone
    td_a = transition_dipoles_uks(A, Ca, Cb, ha, vmin - 1, vmin, cmax, X[:na])
    ref_a = oracle_td(A, Ca, vmin, ha - vmin + 1, ha + 1, cmax - ha, X[:na], prefactor=-1.0)
    assert np.abs(td_a - ref_a).max() <= 1e-12 * np.abs(ref_a).max()


def test_errors():
    from votca_gb300 import _lib
    from votca_gb300.bse import transition_dipoles

    A = np.zeros((3, 5, 5))
    C = np.eye(5)
    with pytest.raises(_lib.BSEError):  # BSE window beyond the orbitals
        transition_dipoles(A, C, homo=2, vmin=0, cmax=7, X=np.zeros((15, 1)))
