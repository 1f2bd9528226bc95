"""Seeded synthetic BSE inputs with the shapes and value distributions of the
VOTCA-XTP GW-BSE workloads this library is measured on.

No public dataset is involved: every array is drawn from a counter-based
generator (splitmix64 of (seed, stream, index), Box-Muller for normals), so a
sub-block can be regenerated without drawing the whole tensor.

Distributions (all energies in eV):
  Mmn[P, m, n] = N(0,1) * 0.1/sqrt(Naux) * exp(-|m-n|/40), symmetric in (m, n)
                 (upper triangle drawn, mirrored)
  occupied QP energies  U[-20, -5], sorted ascending
  virtual QP energies   U[0.5, 30], sorted ascending
  screening: eps = Q diag(lambda) Q^T with lambda ~ U[1, 10]; W = I - eps^-1.
             In the eigenbasis of eps this is w_P = 1 - 1/lambda_P applied to
             M.Q; an orthogonal rotation of iid Gaussian aux-vectors is again iid
             Gaussian with the same variance, so the rotated tensor is drawn
             directly and w is returned as the diagonal screening vector
             (the reference's epsilon_0_inv slot, bse.cc:61-78).
             dense_screening() also returns the dense SPD eps for the Cholesky
             route at small sizes.
"""
from __future__ import annotations

import numpy as np

_M64 = np.uint64(0xFFFFFFFFFFFFFFFF)


def _splitmix(x):
    x = (x + np.uint64(0x9E3779B97F4A7C15)) & _M64
    z = x
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & _M64
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & _M64
    return z ^ (z >> np.uint64(31))


def _uniform(seed, stream, idx):
    with np.errstate(over="ignore"):
        base = _splitmix(np.uint64(seed) * np.uint64(0x100000001B3) + np.uint64(stream))
        h = _splitmix(base ^ idx.astype(np.uint64))
    return ((h >> np.uint64(11)).astype(np.float64) + 0.5) * (1.0 / 9007199254740992.0)


def _normal(seed, stream, idx):
    u1 = _uniform(seed, 2 * stream, idx)
    u2 = _uniform(seed, 2 * stream + 1, idx)
    return np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * np.pi * u2)


def mmn_tensor(seed, naux, nmo, dtype=np.float64):
    """Mmn as (nmo, naux, nmo): M(m, n, P) = out[m, P, n] (reference slice layout)."""
    m = np.arange(nmo)
    lo = np.minimum(m[:, None], m[None, :])
    hi = np.maximum(m[:, None], m[None, :])
    decay = np.exp(-np.abs(m[:, None] - m[None, :]) / 40.0) * (0.1 / np.sqrt(naux))
    out = np.empty((nmo, naux, nmo), dtype=dtype)
    for P in range(naux):
        idx = (np.uint64(P) * np.uint64(nmo) + lo.astype(np.uint64)) * np.uint64(nmo) + hi.astype(np.uint64)
        out[:, P, :] = _normal(seed, 1, idx) * decay
    return out


def mmn_tensor_torch(seed, naux, nmo):
    """Same distribution as mmn_tensor, drawn with torch's seeded generator on
    the GPU when one is present (large sizes).  Each aux slice is a symmetric
    N(0,1) matrix ((G + G^T)/sqrt(2) off the diagonal, G_mm on it) times
    0.1/sqrt(Naux) exp(-|m-n|/40).  Layout (m, P, n), float64 host array (a view of a
    page-locked torch tensor when a GPU is present)."""
    import torch

    dev = "cuda" if torch.cuda.is_available() else "cpu"
    g = torch.Generator(device=dev).manual_seed(int(seed))
    m = torch.arange(nmo, dtype=torch.float64, device=dev)
    decay = torch.exp(-(m[:, None] - m[None, :]).abs() / 40.0) * (0.1 / np.sqrt(naux))
    # page-locked when a GPU is present: the operator staging then copies at full link speed
    out = torch.empty((nmo, naux, nmo), dtype=torch.float64, pin_memory=torch.cuda.is_available())
    chunk = 128
    for p0 in range(0, naux, chunk):
        p1 = min(naux, p0 + chunk)
        G = torch.randn((p1 - p0, nmo, nmo), generator=g, dtype=torch.float64, device=dev)
        M = (G + G.transpose(1, 2)) * (1.0 / np.sqrt(2.0))
        M.diagonal(dim1=1, dim2=2).copy_(G.diagonal(dim1=1, dim2=2))
        out[:, p0:p1, :] = (M * decay).permute(1, 0, 2).cpu()
    return out.numpy()


def qp_energies(seed, v, c):
    occ = np.sort(-20.0 + 15.0 * _uniform(seed, 11, np.arange(v, dtype=np.uint64)))
    virt = np.sort(0.5 + 29.5 * _uniform(seed, 12, np.arange(c, dtype=np.uint64)))
    return np.concatenate([occ, virt])


def screening_eigenvalues(seed, naux):
    return 1.0 + 9.0 * _uniform(seed, 13, np.arange(naux, dtype=np.uint64))


def screening_w(seed, naux):
    """w_P = 1 - 1/lambda_P: W = I - eps^-1 in eps's eigenbasis."""
    return 1.0 - 1.0 / screening_eigenvalues(seed, naux)


def dense_screening(seed, naux):
    """Dense SPD eps = Q diag(lambda) Q^T (Q from QR of a seeded Gaussian) and its
    eigen-pair; for the Cholesky route checks at small naux."""
    lam = screening_eigenvalues(seed, naux)
    G = _normal(seed, 14, np.arange(naux * naux, dtype=np.uint64)).reshape(naux, naux)
    Q, R = np.linalg.qr(G)
    Q = Q * np.sign(np.diag(R))
    eps = (Q * lam) @ Q.T
    return 0.5 * (eps + eps.T), Q, lam


class Problem:
    """One synthetic TDA/full BSE problem.  The BSE window covers MOs
    [0, v + c); extra MOs (nmo > v + c) sit above cmax (rpamax > cmax)."""

    def __init__(self, v, c, naux, nmo=None, seed=0):
        self.v, self.c, self.naux = int(v), int(c), int(naux)
        self.nmo = int(nmo if nmo is not None else v + c)
        self.seed = int(seed)
        self.mmn = mmn_tensor(seed, self.naux, self.nmo)
        e = qp_energies(seed, self.v, self.c)
        self.hqp = np.diag(e)
        self.w = screening_w(seed, self.naux)
        self.dim = self.v * self.c
        self.voff = 0
        self.coff = self.v


class UKSProblem:
    """One synthetic unrestricted problem: alpha and beta channels with their own HOMO over
    MOs [vmin, cmax] of a window starting at rpamin = 0 (nmo MOs, extra MOs above cmax).
    The beta Mmn is drawn from seed + 7919 so that the two channels differ; with
    symmetric=False the (m, n) symmetry is broken by a second draw of the lower triangle
    (exercises which of M(m, n) and M(n, m) each product reads)."""

    def __init__(self, homo_alpha, homo_beta, vmin, cmax, naux, nmo=None, seed=0, symmetric=True):
        self.homo_alpha, self.homo_beta = int(homo_alpha), int(homo_beta)
        self.vmin, self.cmax, self.naux = int(vmin), int(cmax), int(naux)
        self.nmo = int(nmo if nmo is not None else cmax + 1)
        self.seed = int(seed)

        def mmn(sd):
            m = mmn_tensor(sd, self.naux, self.nmo)
            if not symmetric:
                low = np.tril(np.ones((self.nmo, self.nmo), dtype=bool), -1)
                other = mmn_tensor(sd + 104729, self.naux, self.nmo)
                m[:, :, :] = np.where(low[:, None, :], other, m)
            return m

        self.mmn_alpha = mmn(seed)
        self.mmn_beta = mmn(seed + 7919)
        self.w = screening_w(seed, self.naux)

        def hqp(homo, sd):
            v, c = homo - self.vmin + 1, self.cmax - homo
            return np.diag(qp_energies(sd, v, c))

        self.hqp_alpha = hqp(self.homo_alpha, seed)
        self.hqp_beta = hqp(self.homo_beta, seed + 7919)


def batched_shapes(n, seed=0):
    """Shapes of n independent molecules: v ~ U{4..32}, c ~ U{32..256},
    Naux ~ U{128..1024}, Nmo = v + c + 8, and a per-molecule seed."""
    idx = np.arange(n, dtype=np.uint64)
    v = 4 + np.floor(_uniform(seed, 21, idx) * 29).astype(int)
    c = 32 + np.floor(_uniform(seed, 22, idx) * 225).astype(int)
    naux = 128 + np.floor(_uniform(seed, 23, idx) * 897).astype(int)
    return [dict(v=int(v[i]), c=int(c[i]), naux=int(naux[i]), nmo=int(v[i] + c[i] + 8),
                 seed=int(seed * 100003 + i + 1)) for i in range(n)]


CONFIGS = {
    # v, c, naux, nmo, roots
    "C0": dict(v=8, c=64, naux=256, nmo=72, roots=10),
    "C1": dict(v=64, c=512, naux=2048, nmo=576, roots=20),
    "C2": dict(v=128, c=1024, naux=4096, nmo=1152, roots=10),
    "C3": dict(molecules=256, roots=5),  # shapes from batched_shapes
}
