"""Seeded synthetic workloads for the energy-representation path.

ERmod publishes no benchmark inputs; the workloads below are built in memory from a
seed, with the shapes the path is specified on:

``soln_small``   solution mode, 6-site methanol-like solute fixed at the box centre in
                 1000 rigid 3-site waters (jittered 10^3 lattice, 31.0 A cube), PME
                 32^3, order 4, cutoff 12 A, Ewald alpha 0.34/A.
``refs_small``   reference-solvent insertion mode, 4000 waters in a 49.3 A cube, the
                 same 6-site solute inserted at 2000 random placements per frame,
                 PME 48^3, ecorr accumulated.
``refs_large``   33,000 waters in a 99.5 A cube, 12-site solute (charges N(0, 0.3) e
                 made neutral, sigma U(2.5, 3.8) A, eps U(0.02, 0.2) kcal/mol),
                 50,000 insertions per frame, PME 96^3.
``soln_adjoint`` 8,000 waters in a 62 A cube with a 16-site solute (solution mode).
``uneven``       16 water systems of 2,000-60,000 waters (log-uniform) at 0.0334/A^3,
                 each with its own 6-40-site solute and 1,000-20,000 insertions.

Waters: O-H 0.9572 A, HOH 104.52 deg, q_O -0.834, q_H +0.417, O sigma 3.1507 A,
eps 0.1521 kcal/mol, H without LJ.  Lattice sites get a uniform +-0.3 A jitter and a
uniform random orientation, redrawn for every frame from (seed, frame).

Solution mode aborts in the reference when any molecule lies beyond the soft region
of the energy coordinate (eng_sft, engproc.F90:999-1005); the solution-mode workloads
therefore draw their waters from the sites of a slightly finer lattice (11^3 for
``soln_small``, 21^3 for ``soln_adjoint``) that lie farther than ``cavity`` A from the
box centre, where the solute sits.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from . import insertion

WATER_CHARGE = np.array([-0.834, 0.417, 0.417])
WATER_EPS = np.array([0.1521, 0.0, 0.0])
WATER_SIG = np.array([3.1507, 0.0, 0.0])
WATER_MASS = np.array([insertion.MASS["O"], insertion.MASS["H"], insertion.MASS["H"]])


def water_body() -> np.ndarray:
    r, th = 0.9572, math.radians(104.52)
    return np.array([[0.0, 0.0, 0.0],
                     [r, 0.0, 0.0],
                     [r * math.cos(th), r * math.sin(th), 0.0]])


def methanol_like():
    """6-site solute: C, H, H, H, O, HO."""
    xyz = np.array([[0.000, 0.000, 0.000],
                    [-0.363, 1.028, 0.000],
                    [-0.363, -0.514, 0.890],
                    [-0.363, -0.514, -0.890],
                    [1.430, 0.000, 0.000],
                    [1.750, 0.905, 0.000]])
    q = np.array([0.145, 0.04, 0.04, 0.04, -0.683, 0.418])
    sig = np.array([3.5, 2.5, 2.5, 2.5, 3.07, 0.0])
    eps = np.array([0.066, 0.03, 0.03, 0.03, 0.17, 0.0])
    mass = np.array([insertion.MASS[e] for e in "CHHHOH"])
    return dict(xyz=xyz, charge=q, sig=sig, eps=eps, mass=mass)


def random_solute(rng: np.random.Generator, nsite: int):
    """Compact rigid solute: self-avoiding random growth, 1.5 A bonds, >= 2.2 A apart."""
    xyz = [np.zeros(3)]
    for _ in range(100000):
        if len(xyz) == nsite:
            break
        ib = int(rng.integers(len(xyz)))
        d = rng.normal(size=3)
        cand = xyz[ib] + 1.5 * d / np.linalg.norm(d)
        dist = np.linalg.norm(np.array(xyz) - cand, axis=1)
        dist[ib] = np.inf  # the bonded parent sits at 1.5 A
        if np.all(dist >= 2.2):
            xyz.append(cand)
    if len(xyz) != nsite:
        raise RuntimeError("random_solute: growth did not converge")
    xyz = np.array(xyz)
    q = rng.normal(0.0, 0.3, nsite)
    q -= q.mean()
    sig = rng.uniform(2.5, 3.8, nsite)
    eps = rng.uniform(0.02, 0.2, nsite)
    mass = np.full(nsite, insertion.MASS["C"])
    return dict(xyz=xyz - xyz.mean(axis=0), charge=q, sig=sig, eps=eps, mass=mass)


_RADICES = (16, 15, 12, 10, 9, 8, 6, 5, 4, 3, 2)


def fft_friendly(n: int) -> int:
    """Smallest grid length >= n that the PME kernels transform best: even (the real rows
    pair into complex ones) and a product of two radices of at most 16 (two shared-memory
    passes per axis; 2^a 3^b 5^c lengths without such a split, like 125, take three)."""
    m = max(int(n), 2)
    while True:
        if m % 2 == 0 and any(m % r == 0 and m // r in _RADICES for r in _RADICES):
            return m
        m += 1


@dataclasses.dataclass
class Workload:
    name: str
    mode: str                 # "soln" or "refs"
    box: float
    nwater: int
    solute: dict
    params: dict
    seed: int
    frames: int
    ins_per_frame: int
    lattice_n: int
    cavity: float = 0.0
    hist: dict = None
    droplet: float = 0.0      # > 0: non-periodic droplet of this radius, centred on the origin

    # ------------------------------------------------------------------
    @property
    def cell(self) -> np.ndarray:
        if self.droplet > 0:  # non-periodic: the cell is not used; a zero cell is passed
            return np.zeros((3, 3))
        return np.diag([self.box] * 3)

    def species(self):
        """MDinfo order: water first, solute last (REFS needs the test particle last)."""
        sl = self.solute
        return [dict(count=self.nwater, sluvid=0, charge=WATER_CHARGE, eps=WATER_EPS, len=WATER_SIG),
                dict(count=1, sluvid=1 if self.mode == "soln" else 2, charge=sl["charge"],
                     eps=sl["eps"], len=sl["sig"])]

    def _lattice_sites(self):
        rng = np.random.default_rng((self.seed, 7))
        n = self.lattice_n
        g = (np.arange(n) + 0.5) * (self.box / n)
        pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
        if self.mode == "soln" and self.cavity > 0:
            c = np.full(3, self.box / 2)
            keep = np.linalg.norm(pts - c, axis=1) > self.cavity
            pts = pts[keep]
        if self.droplet > 0:
            keep = np.linalg.norm(pts - np.full(3, self.box / 2), axis=1) < self.droplet
            pts = pts[keep]
        if len(pts) > self.nwater:
            pick = np.sort(rng.choice(len(pts), self.nwater, replace=False))
            pts = pts[pick]
        assert len(pts) == self.nwater, (len(pts), self.nwater)
        return pts

    def frame(self, i: int):
        """(sitepos (numatm, 3), cell) for frame i."""
        if not hasattr(self, "_lat"):
            self._lat = self._lattice_sites()
        rng = np.random.default_rng((self.seed, 1000 + i))
        n = self.nwater
        centres = self._lat + rng.uniform(-0.3, 0.3, (n, 3))
        q = insertion.random_quaternions(rng, n)
        body = water_body()
        body = body - insertion.center_of_mass(body, WATER_MASS)
        wat = insertion.quat_rotate(q, np.broadcast_to(body, (n, 3, 3))) + centres[:, None, :]
        sl = self.solute["xyz"] - insertion.center_of_mass(self.solute["xyz"], self.solute["mass"])
        sl = sl + self.box / 2
        pos = np.concatenate([wat.reshape(-1, 3), sl], axis=0)
        if self.droplet > 0:
            pos = pos - self.box / 2
        return np.ascontiguousarray(pos), self.cell

    def placements(self, i: int, n: int = None):
        """REFS: (n, nsite, 3) solute coordinates of frame i's insertions."""
        n = self.ins_per_frame if n is None else n
        rng = np.random.default_rng((self.seed, 500000 + i))
        return insertion.random_placements(rng, self.solute["xyz"], self.solute["mass"], self.cell, n)

    @property
    def units_per_frame(self) -> int:
        return self.ins_per_frame * self.nwater


def _params(slttype, K, corrcal, wgtslf, estype=2, screen=0.34, temp_K=300.0):
    return dict(slttype=slttype, estype=estype, ljswitch=0, splodr=4, ms1max=K, ms2max=K, ms3max=K,
                wgtslf=wgtslf, corrcal=corrcal, selfcal=0, force_calculation=0,
                elecut=12.0, lwljcut=10.0, upljcut=12.0, screen=screen,
                temp=temp_K * 8.314510e-3 / 4.184, block_threshold=4.0)


def soln_small(seed: int = 1, frames: int = 100) -> Workload:
    return Workload("soln_small", "soln", 31.0, 1000, methanol_like(),
                    _params(1, 32, corrcal=0, wgtslf=0), seed, frames, 1, 11, cavity=4.5)


def refs_small(seed: int = 2, frames: int = 50, ins: int = 2000) -> Workload:
    return Workload("refs_small", "refs", 49.3, 4000, methanol_like(),
                    _params(2, 48, corrcal=1, wgtslf=1), seed, frames, ins, 16)


def refs_large(seed: int = 3, frames: int = 20, ins: int = 50000) -> Workload:
    rng = np.random.default_rng((seed, 11))
    return Workload("refs_large", "refs", 99.5, 33000, random_solute(rng, 12),
                    _params(2, 96, corrcal=1, wgtslf=1), seed, frames, ins, 33)


def droplet(seed: int = 6, frames: int = 20) -> Workload:
    """Non-periodic (boxshp 0) water droplet of radius 13 A around the methanol-like
    solute, centred on the origin: bare Coulomb without cutoff, NVT."""
    p = _params(1, 32, corrcal=0, wgtslf=0, estype=1)
    p.update(cltype=0, boxshp=0)
    return Workload("droplet", "soln", 31.0, 300, methanol_like(), p, seed, frames, 1, 11, cavity=4.5,
                    droplet=13.0)


def soln_adjoint(seed: int = 5, frames: int = 200) -> Workload:
    rng = np.random.default_rng((seed, 11))
    # a 7.5 A cavity around the 4.2 A solute: with 6.0 A a water of some frames (frame 7
    # of seed 5) comes within 2.5 A of a solute site, where the reference stops (eng_sft)
    return Workload("soln_adjoint", "soln", 62.0, 8000, random_solute(rng, 16),
                    _params(1, 64, corrcal=0, wgtslf=0), seed, frames, 1, 21, cavity=7.5)


def uneven(seed: int = 4):
    """16 systems, log-uniform 2k-60k waters at 0.0334 / A^3."""
    rng = np.random.default_rng((seed, 13))
    out = []
    for s in range(16):
        n = int(round(math.exp(rng.uniform(math.log(2000), math.log(60000)))))
        box = (n / 0.0334) ** (1.0 / 3.0)
        nsite = int(rng.integers(6, 41))
        ins = int(rng.integers(1000, 20001))
        K = fft_friendly(int(math.ceil(box / 1.0)))
        lat = int(math.ceil(n ** (1.0 / 3.0)))
        sol = random_solute(rng, nsite)
        # gen_input's --minenergy: solutes of up to 40 charged sites bind some waters
        # below the default -20 kcal/mol first edge, which the reference stops on (eng_min)
        hist = dict(ecdmin=-200.0, ecfmns=-0.20, ecdcen=0.0, eccore=20.0, ecdmax=1.0e11,
                    eclbin=5.0e-2, ecfbin=2.0e-3, ec0bin=2.0e-4, finfac=10.0, pecore=200)
        out.append(Workload(f"uneven_{s}", "refs", box, n, sol, _params(2, K, corrcal=1, wgtslf=1),
                            seed * 100 + s, 1, ins, lat, hist=hist))
    return out


WORKLOADS = {"soln_small": soln_small, "refs_small": refs_small, "refs_large": refs_large,
             "soln_adjoint": soln_adjoint}
