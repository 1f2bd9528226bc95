"""Regenerates the golden fixtures in this folder from the VOTCA-XTP test data.

Run where the reference tree (votca/votca) is available, giving its root as the argument or
in the environment variable VOTCA_REFERENCE_ROOT:
    python tests/golden/make_golden.py REF

Writes bse_operator_hqp.npz:
  Hqp      17x17  xtp/src/tests/DataFiles/bse_operator/Hqp.mm   (operator input)
  hqp_ref  20x20  xtp/src/tests/DataFiles/bse_operator/hqp_ref.mm
           (HqpOperator * Identity for homo=4, vmin=0, cmax=8, qpmin=rpamin=0;
            xtp/src/tests/test_bse_operator.cc:74-93, compared at isApprox 1e-3)
  epsilon_inv 17  the screening vector hard-coded at test_bse_operator.cc:65-72
Writes davidson_kat.npz: the lowest 10 eigenvalues of init_matrix(N, 0.01)
(test_davidson.cc:42-56) for N = 100, 400, from a dense symmetric eigensolver,
the reference value its Davidson tests check against at 1e-6.
Writes bse_operator_methane.npz (xtp/src/tests/DataFiles/bse_operator and .../bse, the inputs
and golden outputs of xtp/src/tests/test_bse_operator.cc:37-147 besides those above):
  basis_xml     the 3-21G basis file (bse/3-21G.xml, used as DFT and auxiliary basis)
  elements, xyz the methane geometry in Angstrom (bse/molecule.xyz)
  MOs           17x17 MO coefficients (bse_operator/MOs.mm)
  rpa_op        17x17 matrix the filled Mmn is multiplied with (bse_operator/rpa_op.mm)
  hx_ref, hd_ref, hd2_ref   HxOperator / HdOperator / Hd2Operator * Identity, 20x20
Writes bse_methane.npz (xtp/src/tests/DataFiles/bse; the inputs and golden outputs of
xtp/src/tests/test_bse.cc:37-330):
  MOs, Hqp                      17x17 MO coefficients and QP Hamiltonian (RPA energies =
                                its diagonal)
  singlets_nooffdiag_tda, singlets_tda, singlets_btda, triplets_tda   lowest roots
  singlets_psi_nooffdiag_tda, singlets_psi_tda, singlets_psi_btda, singlets_psi_AR_btda,
  triplets_psi_tda              eigenvectors (the reference compares subspace projections)
  singlets_dynamic_TDA, singlets_dynamic_full, triplets_dynamic_TDA   perturbative dynamical
                                screening
Writes rpa_methane.npz (xtp/src/tests/DataFiles/rpa; xtp/src/tests/test_rpa.cc:69-140 checks at
isApprox 1e-4):
  eigenvectors, eigenvals   MO coefficients and RPA input energies (same molecule and basis)
  r_ref, r_complex_ref      RPA::calculate_epsilon_r at 0 and at 0.5 + 0.5i (homo 4, rpa 0..16)
Writes threecenter_gwbse.npz (xtp/src/tests/DataFiles/threecenter_gwbse, the same methane
geometry and 3-21G basis; checked by xtp/src/tests/test_threecenter_gwbse.cc:36-123 at
isApprox 1e-5):
  MOs                17x17 MO coefficients
  ref0b, ref2b, ref4b  slices m = 0, 2, 4 (8 x 17: n = 0..7 by aux) of TCMatrix_gwbse::Fill
                     over the window m 0..5, n 0..7
Writes orbitals_osc.npz (xtp/src/tests/DataFiles/orbitals and .../aomatrix3d, methane 3-21G):
  basis_xml, elements, xyz   the basis and geometry (orbitals/3-21G.xml, molecule.xyz)
  MOs, spsi                  MOs3.mm and spsi_ref2.mm, the inputs of the osc_strength test
  omega, dipoles_ref, oscs_ref  its literals (test_orbitals.cc:216-250)
  dip_ref, dip_ref_nonzero   AODipole matrices about the origin and about dip_center_nonzero
                             (test_aomatrix3d.cc:36-90)
Writes aomatrix.npz (xtp/src/tests/DataFiles/aomatrix, methane 3-21G; checked by
xtp/src/tests/test_aomatrix.cc:43-123 at isApprox 1e-5):
  overlap, coulomb                 AOOverlap / AOCoulomb matrices (overlap_ref.mm, coulomb_ref.mm)
  invsqrt                          coulomb.Pseudo_InvSqrt(1e-7)          (coulombinvsqrt_ref.mm)
  invsqrt_gwbse                    coulomb.Pseudo_InvSqrt_GWBSE(overlap, 1e-7) (coulombinvsqrtgw_ref.mm)
"""
import os
import sys

import numpy as np


def read_mm_array(path):
    with open(path) as f:
        lines = [l.strip() for l in f if l.strip() and not l.startswith("%")]
    r, c = (int(x) for x in lines[0].split())
    vals = np.array([float(x) for x in lines[1 : 1 + r * c]])
    return vals.reshape(c, r).T.copy()  # column-major storage


def main():
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VOTCA_REFERENCE_ROOT")
    if not ref:
        sys.exit("usage: make_golden.py REF (the votca/votca source root), or set VOTCA_REFERENCE_ROOT")
    here = os.path.dirname(os.path.abspath(__file__))
    d = os.path.join(ref, "xtp/src/tests/DataFiles/bse_operator")
    eps_inv = np.array([
        0.999807798016267, 0.994206065211371, 0.917916768047073, 0.902913813951883,
        0.902913745974602, 0.902913584797742, 0.853352878674581, 0.853352727016914,
        0.853352541699637, 0.79703468058566, 0.797034577207669, 0.797034400395582,
        0.787701833916331, 0.518976361745313, 0.518975064844033, 0.518973712898761,
        0.459286057710524])
    np.savez(os.path.join(here, "bse_operator_hqp.npz"),
             Hqp=read_mm_array(os.path.join(d, "Hqp.mm")),
             hqp_ref=read_mm_array(os.path.join(d, "hqp_ref.mm")),
             epsilon_inv=eps_inv)
    sys.path.insert(0, os.path.join(here, "..", ".."))
    from oracle.davidson_oracle import init_matrix
    out = {}
    for n in (100, 400):
        out[f"evals_{n}"] = np.linalg.eigvalsh(init_matrix(n, 0.01))[:10]
    np.savez(os.path.join(here, "davidson_kat.npz"), **out)
    b = os.path.join(ref, "xtp/src/tests/DataFiles/bse")
    elements, xyz = [], []
    for line in open(os.path.join(b, "molecule.xyz")).read().splitlines()[2:]:
        t = line.split()
        if len(t) == 4:
            elements.append(t[0])
            xyz.append([float(x) for x in t[1:]])
    np.savez(os.path.join(here, "bse_operator_methane.npz"),
             basis_xml=np.array(open(os.path.join(b, "3-21G.xml")).read()),
             elements=np.array(elements), xyz=np.array(xyz),
             MOs=read_mm_array(os.path.join(d, "MOs.mm")),
             rpa_op=read_mm_array(os.path.join(d, "rpa_op.mm")),
             hx_ref=read_mm_array(os.path.join(d, "hx_ref.mm")),
             hd_ref=read_mm_array(os.path.join(d, "hd_ref.mm")),
             hd2_ref=read_mm_array(os.path.join(d, "hd2_ref.mm")))
    keys = ["singlets_nooffdiag_tda", "singlets_tda", "singlets_btda", "triplets_tda",
            "singlets_psi_nooffdiag_tda", "singlets_psi_tda", "singlets_psi_btda",
            "singlets_psi_AR_btda", "triplets_psi_tda", "singlets_dynamic_TDA",
            "singlets_dynamic_full", "triplets_dynamic_TDA"]
    arrays = {k: read_mm_array(os.path.join(b, k + ".mm")) for k in keys}
    for k in keys:
        if "psi" not in k:
            arrays[k] = arrays[k].reshape(-1)
    np.savez(os.path.join(here, "bse_methane.npz"), MOs=read_mm_array(os.path.join(b, "MOs.mm")),
             Hqp=read_mm_array(os.path.join(b, "Hqp.mm")), **arrays)
    r = os.path.join(ref, "xtp/src/tests/DataFiles/rpa")
    np.savez(os.path.join(here, "rpa_methane.npz"),
             eigenvectors=read_mm_array(os.path.join(r, "eigenvectors.mm")),
             eigenvals=read_mm_array(os.path.join(r, "eigenvals.mm")).reshape(-1),
             r_ref=read_mm_array(os.path.join(r, "r_ref.mm")),
             r_complex_ref=read_mm_array(os.path.join(r, "r_complex_ref.mm")))
    t = os.path.join(ref, "xtp/src/tests/DataFiles/threecenter_gwbse")
    np.savez(os.path.join(here, "threecenter_gwbse.npz"),
             MOs=read_mm_array(os.path.join(t, "MOs.mm")),
             ref0b=read_mm_array(os.path.join(t, "ref0b.mm")),
             ref2b=read_mm_array(os.path.join(t, "ref2b.mm")),
             ref4b=read_mm_array(os.path.join(t, "ref4b.mm")))
    a = os.path.join(ref, "xtp/src/tests/DataFiles/aomatrix")
    np.savez(os.path.join(here, "aomatrix.npz"),
             overlap=read_mm_array(os.path.join(a, "overlap_ref.mm")),
             coulomb=read_mm_array(os.path.join(a, "coulomb_ref.mm")),
             invsqrt=read_mm_array(os.path.join(a, "coulombinvsqrt_ref.mm")),
             invsqrt_gwbse=read_mm_array(os.path.join(a, "coulombinvsqrtgw_ref.mm")))
    write_orbitals_osc(ref, here)
    print("wrote fixtures to", here)


def write_orbitals_osc(ref, here):
    """orbitals_osc.npz: the inputs and golden outputs of the oscillator-strength test
    (xtp/src/tests/test_orbitals.cc:202-256, isApprox 1e-5) and of the AO dipole matrices
    (xtp/src/tests/test_aomatrix3d.cc:36-90, isApprox 1e-4), methane in 3-21G."""
    o = os.path.join(ref, "xtp/src/tests/DataFiles/orbitals")
    a = os.path.join(ref, "xtp/src/tests/DataFiles/aomatrix3d")
    with open(os.path.join(o, "molecule.xyz")) as f:
        lines = f.read().split("\n")
    nat = int(lines[0])
    atoms = [l.split() for l in lines[2:2 + nat]]
    with open(os.path.join(o, "3-21G.xml")) as f:
        basis_xml = f.read()
    # the test's literals: BSE singlet energies, transition dipoles and oscillator strengths for
    # homo = 3 (setNumberOfOccupiedLevels(4)), BSE levels 0..16, TDA
    omega = np.array([0.107455, 0.107455, 0.107455])
    dipoles_ref = np.array([[0.110512, 0.048776, -0.0515914],
                            [-0.13408, 0.0969472, 0.0261392],
                            [0.0586073, 0.121606, -0.0606862]])
    oscs_ref = np.array([0.001236, 0.00201008, 0.00156925])
    np.savez(os.path.join(here, "orbitals_osc.npz"),
             basis_xml=basis_xml, elements=np.array([t[0] for t in atoms]),
             xyz=np.array([[float(x) for x in t[1:4]] for t in atoms]),
             MOs=read_mm_array(os.path.join(o, "MOs3.mm")),
             spsi=read_mm_array(os.path.join(o, "spsi_ref2.mm")),
             omega=omega, dipoles_ref=dipoles_ref, oscs_ref=oscs_ref,
             dip_ref=np.array([read_mm_array(os.path.join(a, f"dip_ref{i}.mm")) for i in range(3)]),
             dip_ref_nonzero=np.array([read_mm_array(os.path.join(a, f"dip_ref{i}_nonzero.mm")) for i in range(3)]),
             dip_center_nonzero=np.array([1.71, 2.34, 3.54]))


if __name__ == "__main__":
    main()
