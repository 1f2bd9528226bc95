"""Gaussian integrals for the reference's small test molecules (TEST INFRASTRUCTURE ONLY).

Only tests/ use this module: it produces the AO inputs (overlap, two- and three-centre Coulomb
integrals) that the reference computes with libint2 (absent here), so that the reference's
golden operator matrices for methane in 3-21G can be reproduced through this repository's Mmn
producer and BSE operator (xtp/src/tests/test_bse_operator.cc:37-147, whose Mmn comes from
TCMatrix_gwbse::Fill with the DFT basis also used as the auxiliary basis).

The integrals follow the published McMurchie-Davidson scheme (J. Comput. Phys. 26, 218 (1978)):
products of Cartesian Gaussians expanded in Hermite Gaussians (E coefficients), Coulomb
integrals from the Hermite auxiliary integrals R_tuv built on the Boys function
F_n(T) = 1F1(n + 1/2; n + 3/2; -T) / (2n + 1).  A three-centre integral (P|mu nu) is the
four-centre formula with a unit s function (exponent 0) beside P; a two-centre one has unit
functions on both sides.  Shells with s and p functions only (what 3-21G needs).

Conventions checked against the reference's golden matrices (tests/test_integrals_golden.py):
primitives normalised, contraction coefficients used as given (the contracted 2s of carbon has
a norm of 1.00001 in overlap_ref.mm), p components in the order the golden overlap shows,
coordinates converted from Angstrom with 1.8897259886 Bohr per Angstrom
(tools/include/votca/tools/constants.h:48).
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET

import numpy as np
from scipy.special import hyp1f1

ANG2BOHR = 1.8897259886
# Cartesian exponents of the p components, in the order the reference's matrices use
P_ORDER = ((0, 1, 0), (0, 0, 1), (1, 0, 0))


def boys(n, T):
    return hyp1f1(n + 0.5, n + 1.5, -T) / (2.0 * n + 1.0)


class Shell:
    def __init__(self, center, l, exps, coefs):
        self.center = np.asarray(center, dtype=np.float64)
        self.l = l
        self.exps = np.asarray(exps, dtype=np.float64)
        self.coefs = np.asarray(coefs, dtype=np.float64)
        comps = [(0, 0, 0)] if l == 0 else list(P_ORDER)
        self.comps = comps

    def size(self):
        return len(self.comps)


def _norm(alpha, lmn):
    l = sum(lmn)
    return (2.0 * alpha / math.pi) ** 0.75 * (4.0 * alpha) ** (l / 2.0)  # (2k-1)!! = 1 for k <= 1


def parse_basis(xml_text):
    """{element: [(type 'S'|'P', [exponents], [coefficients])]}, SP shells split in S and P."""
    root = ET.fromstring(xml_text)
    out = {}
    for el in root.findall("element"):
        shells = []
        for sh in el.findall("shell"):
            types = sh.get("type")
            prims = sh.findall("constant")
            for t in types:
                exps, cfs = [], []
                for c in prims:
                    for con in c.findall("contractions"):
                        if con.get("type") == t:
                            exps.append(float(c.get("decay")))
                            cfs.append(float(con.get("factor")))
                shells.append((t, exps, cfs))
        out[el.get("name")] = shells
    return out


def build_shells(atoms, basis):
    """atoms: [(element, (x, y, z) in Angstrom)] in file order."""
    shells = []
    for el, xyz in atoms:
        c = np.asarray(xyz, dtype=np.float64) * ANG2BOHR
        for t, exps, cfs in basis[el]:
            shells.append(Shell(c, 0 if t == "S" else 1, exps, cfs))
    return shells


def _E(i, j, t, Qx, a, b):
    """Hermite expansion coefficient of x_A^i x_B^j exp(-a x_A^2 - b x_B^2), Qx = A - B."""
    p = a + b
    q = a * b / p
    if t < 0 or t > i + j:
        return 0.0
    if i == 0 and j == 0 and t == 0:
        return math.exp(-q * Qx * Qx)
    if j == 0:
        return (_E(i - 1, j, t - 1, Qx, a, b) / (2 * p) - (q * Qx / a) * _E(i - 1, j, t, Qx, a, b)
                + (t + 1) * _E(i - 1, j, t + 1, Qx, a, b))
    return (_E(i, j - 1, t - 1, Qx, a, b) / (2 * p) + (q * Qx / b) * _E(i, j - 1, t, Qx, a, b)
            + (t + 1) * _E(i, j - 1, t + 1, Qx, a, b))


def _R_table(L, alpha, PC):
    """R_tuv (t + u + v <= L) of the Hermite Coulomb integrals at exponent alpha, separation PC."""
    T = alpha * float(PC @ PC)
    F = [boys(n, T) for n in range(L + 1)]
    memo = {}

    def R(t, u, v, n):
        key = (t, u, v, n)
        if key in memo:
            return memo[key]
        if t < 0 or u < 0 or v < 0:
            return 0.0
        if t == 0 and u == 0 and v == 0:
            val = (-2.0 * alpha) ** n * F[n]
        elif t == 0 and u == 0:
            val = (v - 1) * R(t, u, v - 2, n + 1) + PC[2] * R(t, u, v - 1, n + 1)
        elif t == 0:
            val = (u - 1) * R(t, u - 2, v, n + 1) + PC[1] * R(t, u - 1, v, n + 1)
        else:
            val = (t - 1) * R(t - 2, u, v, n + 1) + PC[0] * R(t - 1, u, v, n + 1)
        memo[key] = val
        return val

    return R


def _pair_hermite(la, A, a, lb, B, b):
    """For every (component of a, component of b): {(t, u, v): E_t E_u E_v}; b = 0 is the unit s."""
    comps_a = [(0, 0, 0)] if la == 0 else list(P_ORDER)
    comps_b = [(0, 0, 0)] if lb == 0 else list(P_ORDER)
    Q = A - B
    out = {}
    for ia, ca in enumerate(comps_a):
        for ib, cb in enumerate(comps_b):
            terms = {}
            ex = [[_E(ca[d], cb[d], t, Q[d], a, b) for t in range(ca[d] + cb[d] + 1)] for d in range(3)]
            for t, et in enumerate(ex[0]):
                for u, eu in enumerate(ex[1]):
                    for v, ev in enumerate(ex[2]):
                        w = et * eu * ev
                        if w != 0.0:
                            terms[(t, u, v)] = w
            out[(ia, ib)] = terms
    return out


def overlap(shells):
    n = sum(s.size() for s in shells)
    S = np.zeros((n, n))
    offs = np.cumsum([0] + [s.size() for s in shells])
    for I, sa in enumerate(shells):
        for J, sb in enumerate(shells):
            for a, da in zip(sa.exps, sa.coefs):
                for b, db in zip(sb.exps, sb.coefs):
                    p = a + b
                    herm = _pair_hermite(sa.l, sa.center, a, sb.l, sb.center, b)
                    for (ia, ib), terms in herm.items():
                        w = terms.get((0, 0, 0), 0.0) * (math.pi / p) ** 1.5
                        S[offs[I] + ia, offs[J] + ib] += (da * db * _norm(a, sa.comps[ia]) * _norm(b, sb.comps[ib])
                                                          * w)
    return S


def dipole(shells, origin=(0.0, 0.0, 0.0)):
    """<mu| r_i - O_i |nu> for i = x, y, z as a (3, n, n) array: the AODipole matrices
    (libint2 emultipole1 about the origin O, xtp/src/libxtp/libint2_calls.cc:206-214).  In the
    Hermite expansion the Cartesian factor is (E_1 + X_PO E_0) (pi/p)^(1/2) along the dipole
    axis and E_0 (pi/p)^(1/2) along the two others (McMurchie-Davidson, as the overlap)."""
    O = np.asarray(origin, dtype=np.float64)
    n = sum(s.size() for s in shells)
    D = np.zeros((3, n, n))
    offs = np.cumsum([0] + [s.size() for s in shells])
    for I, sa in enumerate(shells):
        for J, sb in enumerate(shells):
            Q = sa.center - sb.center
            for a, da in zip(sa.exps, sa.coefs):
                for b, db in zip(sb.exps, sb.coefs):
                    p = a + b
                    P = (a * sa.center + b * sb.center) / p
                    for ia, ca in enumerate(sa.comps):
                        for ib, cb in enumerate(sb.comps):
                            e0 = [_E(ca[d], cb[d], 0, Q[d], a, b) for d in range(3)]
                            e1 = [_E(ca[d], cb[d], 1, Q[d], a, b) for d in range(3)]
                            f = da * db * _norm(a, ca) * _norm(b, cb) * (math.pi / p) ** 1.5
                            for k in range(3):
                                w = e1[k] + (P[k] - O[k]) * e0[k]
                                for d in range(3):
                                    if d != k:
                                        w *= e0[d]
                                D[k, offs[I] + ia, offs[J] + ib] += f * w
    return D


def _eri(bra, ket, p, q, Pc, Qc):
    """sum over Hermite terms of bra (dict) and ket (dict) with the (-1)^(ket order) sign."""
    alpha = p * q / (p + q)
    L = max(sum(k) for k in bra) + max(sum(k) for k in ket)
    R = _R_table(L, alpha, Pc - Qc)
    s = 0.0
    for (t, u, v), eb in bra.items():
        for (tt, uu, vv), ek in ket.items():
            s += eb * ek * (-1.0) ** (tt + uu + vv) * R(t + tt, u + uu, v + vv, 0)
    return 2.0 * math.pi ** 2.5 / (p * q * math.sqrt(p + q)) * s


def coulomb2(shells):
    """(P|Q) = integral of phi_P(1) phi_Q(2) / r12."""
    n = sum(s.size() for s in shells)
    V = np.zeros((n, n))
    offs = np.cumsum([0] + [s.size() for s in shells])
    for I, sa in enumerate(shells):
        for J, sb in enumerate(shells):
            for a, da in zip(sa.exps, sa.coefs):
                ha = _pair_hermite(sa.l, sa.center, a, 0, sa.center, 0.0)
                for b, db in zip(sb.exps, sb.coefs):
                    hb = _pair_hermite(sb.l, sb.center, b, 0, sb.center, 0.0)
                    for ia in range(sa.size()):
                        for ib in range(sb.size()):
                            v = _eri(ha[(ia, 0)], hb[(ib, 0)], a, b, sa.center, sb.center)
                            V[offs[I] + ia, offs[J] + ib] += (da * db * _norm(a, sa.comps[ia])
                                                              * _norm(b, sb.comps[ib]) * v)
    return V


def coulomb3(aux, ao):
    """(P|mu nu) as an (naux, nao, nao) array."""
    naux = sum(s.size() for s in aux)
    nao = sum(s.size() for s in ao)
    out = np.zeros((naux, nao, nao))
    oa = np.cumsum([0] + [s.size() for s in aux])
    ob = np.cumsum([0] + [s.size() for s in ao])
    for K, sc in enumerate(aux):
        for I, sa in enumerate(ao):
            for J, sb in enumerate(ao):
                if J < I:
                    continue
                blk = np.zeros((sc.size(), sa.size(), sb.size()))
                for c, dc in zip(sc.exps, sc.coefs):
                    hc = _pair_hermite(sc.l, sc.center, c, 0, sc.center, 0.0)
                    for a, da in zip(sa.exps, sa.coefs):
                        for b, db in zip(sb.exps, sb.coefs):
                            q = a + b
                            Qc = (a * sa.center + b * sb.center) / q
                            hab = _pair_hermite(sa.l, sa.center, a, sb.l, sb.center, b)
                            for ic in range(sc.size()):
                                for (ia, ib), terms in hab.items():
                                    v = _eri(hc[(ic, 0)], terms, c, q, sc.center, Qc)
                                    blk[ic, ia, ib] += (dc * da * db * _norm(c, sc.comps[ic])
                                                        * _norm(a, sa.comps[ia]) * _norm(b, sb.comps[ib]) * v)
                out[oa[K]:oa[K + 1], ob[I]:ob[I + 1], ob[J]:ob[J + 1]] = blk
                out[oa[K]:oa[K + 1], ob[J]:ob[J + 1], ob[I]:ob[I + 1]] = blk.transpose(0, 2, 1)
    return out
