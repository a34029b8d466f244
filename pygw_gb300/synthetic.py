"""Seeded synthetic inputs for the polarization path (weights → χ0 → ε⁻¹).

No crystal, WIEN2k case or public dataset is involved: every array is
generated from a seed with the shapes and value distributions of the five
workloads the project measures on.

* Bands: cubic tight-binding ``E_n(k) = −2t(cos kx + cos ky + cos kz) + 0.8·n``
  eV, t = 1 eV, ``k_i = 2π j_i / n`` on a Γ-centred n³ mesh, plus Gaussian
  jitter σ = 0.1 eV drawn per (k, n) from ``numpy.random.default_rng(seed)``.
* Fermi level mid-gap between the band centres of n = nocc−1 and nocc:
  ``EF = 0.8·(nocc − 0.5)`` eV.
* Band windows by PyGW's rule (pygw.py:999-1009): ``nomx = max_k nocc(k) − 1``,
  ``numin = min_k nocc(k)``; ``nbmaxpol`` = all bands, no core states
  (``ncg = 0``).
* Matsubara frequencies: log-spaced.
* Coulomb: ``v_I = 4π/|q+G_I|²`` with ``|q+G_I|`` uniform in 0.5–8 bohr⁻¹.
* Matrix elements ``M_{p,I}(k) ~ CN(0,1)/(1+|E_n(k)−E_m(k−q)|)·√v_I`` complex128,
  generated per k from ``(seed, q, k)`` so any k-chunk can be regenerated
  independently.  The ``√v_I`` factor is the diagonal ``barcvm`` of the
  reference (``minm = mmat·conj(barcvm)``, pygw.py:2666).
* q→0 wings: ``pm_p(k) ~ CN(0,1)/(1+|ΔE|)``; head from the same tetrahedron
  weights (``head(ω) = −2 Σ_k Σ_p |pm_p(k)|² w_p(k,ω)``), kept in FP64.

Energies stay in eV end to end, so weights are in 1/eV.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from .mesh import KQmesh, kpoint_coords


@dataclass(frozen=True)
class Workload:
    name: str
    div: int                 # n of the n×n×n Γ-centred mesh
    nbands: int
    nocc: int
    npb: int                 # product-basis size N_PB
    nom: int
    om_lo: float
    om_hi: float
    nq: int
    seed: int = 0
    t_hop: float = 1.0
    spacing: float = 0.8
    jitter: float = 0.1
    npb_range: tuple = field(default=())  # uneven N_PB per q (batched workload)


WORKLOADS = {
    # 4³ k, 32 bands (8 occ), N_PB=128, 16 ω in 0.01–100 eV, one q
    "C1": Workload("C1", 4, 32, 8, 128, 16, 0.01, 100.0, 1),
    # 8³ k, 60 bands (4 occ), N_PB=400, 32 ω, 10 q
    "C2": Workload("C2", 8, 60, 4, 400, 32, 0.01, 100.0, 10),
    # 6³ k, 200 bands (16 occ), N_PB=1200, 48 ω, 8 q
    "C3": Workload("C3", 6, 200, 16, 1200, 48, 0.01, 100.0, 8),
    # 6³ k, 48 ω, 20 q with N_PB uniform in 600–1500 per q
    "C4": Workload("C4", 6, 300, 16, 1200, 48, 0.01, 100.0, 20, npb_range=(600, 1500)),
    # 10³ k, 400 bands (32 occ), N_PB=2000, 64 ω in 0.005–200 eV, 4 q incl. q→0
    "C5": Workload("C5", 10, 400, 32, 2000, 64, 0.005, 200.0, 4),
}


def scaled(w: Workload, **kw) -> Workload:
    """Copy of a workload with some fields replaced (small test cases)."""
    d = dict(w.__dict__)
    d.update(kw)
    return Workload(**d)


class Bands:
    """Band energies and the reference's band-window bookkeeping.

    Attributes mirror what ``Polarization_weights`` reads from the
    Kohn–Sham object: ``Ebnd[isp, irk, n]`` (relative to nothing: EF is
    passed separately), ``EF``, ``nomax_numin``, ``ncg_p``, ``nbmaxpol``.
    """

    def __init__(self, w: Workload, kqm: KQmesh):
        self.w = w
        rng = np.random.default_rng(w.seed)
        kf = kpoint_coords(kqm.ndiv) * 2.0 * np.pi
        disp = -2.0 * w.t_hop * np.cos(kf).sum(axis=1)                    # [nkp]
        e = disp[:, None] + w.spacing * np.arange(w.nbands)[None, :]
        e = e + w.jitter * rng.standard_normal((kqm.nkp, w.nbands))
        self.Ebnd = e[None, :, :].copy()                                  # [nspin=1, nkp, nband]
        self.EF = w.spacing * (w.nocc - 0.5)
        nocc_at_k = (e < self.EF).sum(axis=1)
        # pygw.py:1003-1009 (energies there are relative to EF, hence x<0)
        self.nomax_numin = [int(nocc_at_k.max()) - 1, int(nocc_at_k.min())]
        self.ncg_p = 0
        self.nbmaxpol = w.nbands

    def enk(self, isp=0):
        """``enk[nbnd, nkp]`` (Fortran order) as assembled at pygw.py:3420-3426."""
        nbnd = self.ncg_p + self.nbmaxpol
        out = np.zeros((nbnd, self.Ebnd.shape[1]), order="F")
        out[self.ncg_p:, :] = self.Ebnd[isp, :, : self.nbmaxpol].T
        return out

    @property
    def nb1(self):
        return self.ncg_p + self.nomax_numin[0] + 1

    @property
    def nb2(self):
        return self.ncg_p + self.nbmaxpol - self.ncg_p - self.nomax_numin[1]


class FrequencyMesh:
    """Matsubara points (``fr.omega``), log-spaced."""

    def __init__(self, w: Workload):
        self.omega = np.geomspace(w.om_lo, w.om_hi, w.nom)


def q_indices(w: Workload, kqm: KQmesh):
    """The q points a workload visits: seeded distinct mesh indices; the first
    is q=0 (Γ, the q→0 head/wings case) for the large workload."""
    rng = np.random.default_rng([w.seed, 7])
    nq = min(w.nq, kqm.nkp)
    if w.name == "C5":
        rest = rng.choice(np.arange(1, kqm.nkp), size=nq - 1, replace=False)
        return [0] + [int(x) for x in rest]
    if nq == 1:
        return [1 % kqm.nkp]
    return [int(x) for x in rng.choice(kqm.nkp, size=nq, replace=False)]


def npb_for_q(w: Workload, iq_pos: int):
    if not w.npb_range:
        return w.npb
    rng = np.random.default_rng([w.seed, 11, iq_pos])
    return int(rng.integers(w.npb_range[0], w.npb_range[1] + 1))


def coulomb_sqrt(w: Workload, iq: int, npb: int):
    """√v_I with v_I = 4π/|q+G_I|², |q+G_I| ~ U(0.5, 8) bohr⁻¹ (seeded per q)."""
    rng = np.random.default_rng([w.seed, 3, iq])
    qg = rng.uniform(0.5, 8.0, size=npb)
    return np.sqrt(4.0 * np.pi / qg ** 2)


def minm_k(w: Workload, bands: Bands, kqm: KQmesh, iq: int, ik: int, sqv):
    """``minm[nb1, nb2, matsiz]`` complex128 for one k (the layout of
    pygw.py:3100-3104, occupied index first)."""
    enk = bands.enk()
    nomx, numin = bands.nomax_numin
    nb1, nb2 = bands.nb1, bands.nb2
    jk = int(kqm.kqid[ik, iq])
    e_n = enk[:nb1, ik]
    e_m = enk[bands.ncg_p + numin: bands.ncg_p + numin + nb2, jk]
    scale = 1.0 / (1.0 + np.abs(e_n[:, None] - e_m[None, :]))          # [nb1, nb2]
    rng = np.random.default_rng([w.seed, 5, iq, ik])
    npb = sqv.shape[0]
    z = rng.standard_normal((nb1, nb2, npb, 2))
    m = (z[..., 0] + 1j * z[..., 1]) * np.sqrt(0.5)
    return m * scale[:, :, None] * sqv[None, None, :]


def pm_k(w: Workload, bands: Bands, ik: int):
    """q→0 wing vector ``pm[ie12]`` for one k, ie12 = ie1*nb2 + ie2 (pygw.py:3120-3141)."""
    enk = bands.enk()
    numin = bands.nomax_numin[1]
    nb1, nb2 = bands.nb1, bands.nb2
    e_n = enk[:nb1, ik]
    e_m = enk[bands.ncg_p + numin: bands.ncg_p + numin + nb2, ik]
    rng = np.random.default_rng([w.seed, 9, ik])
    z = rng.standard_normal((nb1, nb2, 2))
    p = (z[..., 0] + 1j * z[..., 1]) * np.sqrt(0.5) / (1.0 + np.abs(e_n[:, None] - e_m[None, :]))
    return p.reshape(-1)


def head_from_weights(kcw, pms):
    """Synthetic q→0 head: ``head(ω) = −2 Σ_k Σ_p |pm_p(k)|² w_p(k,ω)`` (FP64),
    the form of calc_head's head sum (pygw.py:2949-3027) without the LAPW
    momentum matrix elements."""
    nb1, nb2, nkp, nom = kcw.shape
    head = np.zeros(nom, dtype=complex)
    for ik in range(nkp):
        a2 = np.abs(pms[ik]) ** 2
        head += -2.0 * (a2[:, None] * kcw[:, :, ik, :].reshape(nb1 * nb2, nom)).sum(axis=0)
    return head


class Problem:
    """Everything one workload needs: mesh, bands, frequencies, q list."""

    def __init__(self, w: Workload):
        self.w = w
        self.kqm = KQmesh((w.div, w.div, w.div))
        self.bands = Bands(w, self.kqm)
        self.fr = FrequencyMesh(w)
        self.qs = q_indices(w, self.kqm)
