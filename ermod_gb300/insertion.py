"""Test-particle placements for reference-solvent (REFS) mode.

Restates the default insertion scheme of ERmod (``insertion.F90``):
``insorigin = 0`` (solute centre of mass moved to the origin, ``set_solute_origin``
insertion.F90:103-131), ``insposition = 0`` (centre of mass translated by
``cell . U[0,1)^3``, insertion.F90:153-163) and ``insorient = 0`` (rotation about the
centre of mass by a unit quaternion drawn by rejection from ``U[-1,1]^4``,
insertion.F90:341-357, applied as ``q v q*`` as in bestfit.F90:75-100).

The reference draws from the Fortran compiler's ``random_number``; that stream is
compiler specific, so placement sequences are not part of parity.  Here the stream
is numpy's PCG64 with a recorded seed, and the GPU path and the oracle consume the
same placements.
"""
from __future__ import annotations

import numpy as np

# getmass (setconf.F90:999-1053)
MASS = {"H": 1.00794, "C": 12.0107, "O": 15.9994, "N": 14.00674, "S": 32.066, "P": 30.973761}


def center_of_mass(xyz: np.ndarray, mass: np.ndarray) -> np.ndarray:
    """bestfit.F90:158-172 -- xyz (..., n, 3)."""
    return np.einsum("...ni,n->...i", xyz, mass) / mass.sum()


def quat_rotate(q: np.ndarray, v: np.ndarray) -> np.ndarray:
    """r = q v q* for unit quaternions q (..., 4) = (w, x, y, z) and vectors v (..., n, 3)."""
    w = q[..., 0][..., None, None]
    u = q[..., 1:][..., None, :]
    t = 2.0 * np.cross(u, v)
    return v + w * t + np.cross(u, t)


def random_quaternions(rng: np.random.Generator, n: int) -> np.ndarray:
    """Rejection sampling of U[-1,1]^4 inside the unit ball, then normalised."""
    out = np.empty((n, 4))
    filled = 0
    while filled < n:
        cand = rng.random((max(16, 4 * (n - filled)), 4)) * 2.0 - 1.0
        cand = cand[np.sum(cand * cand, axis=1) < 1.0]
        take = min(len(cand), n - filled)
        out[filled:filled + take] = cand[:take]
        filled += take
    return out / np.linalg.norm(out, axis=1, keepdims=True)


def random_placements(rng: np.random.Generator, bfcoord: np.ndarray, mass: np.ndarray,
                      cell: np.ndarray, n: int) -> np.ndarray:
    """n placements of a rigid solute -> (n, nsite, 3) site coordinates."""
    body = bfcoord - center_of_mass(bfcoord, mass)           # COM to the origin
    r = rng.random((n, 3))
    com = r @ cell.T                                           # cell . r
    q = random_quaternions(rng, n)
    rot = quat_rotate(q, np.broadcast_to(body, (n,) + body.shape))
    return rot + com[:, None, :]
