"""Set-up semantics of the reference, computed through the library's host helpers.

* ``setparam_topology``: engmain's topology state from per-species site tables
  (LJ-type deduplication and combination rules, setconf.F90:720-823, via
  ``ermod_lj_tables``; charge scaling setconf.F90:829; molecular charges
  setconf.F90:832-834; the species numbering ``uvspec`` of engproc.F90:102-120).
* ``enginit_bins``: the energy coordinate of enginit (engproc.F90:122-237, via
  ``ermod_enginit_species``).
* ``getscrn``: the Ewald screening parameter from ``ewtoler`` (setconf.F90:515-535).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib

CHARGE_SCALE = 18.22261721  # sqrt(e^2 N_A / (4 pi eps0) / (kcal/mol A)), setconf.F90:829

HIST_DEFAULT = dict(ecdmin=-20.0, ecfmns=-0.20, ecdcen=0.0, eccore=20.0, ecdmax=1.0e11,
                    eclbin=5.0e-2, ecfbin=2.0e-3, ec0bin=2.0e-4, finfac=10.0, pecore=200)


def getscrn(ewtoler: float, elecut: float, distance_form: bool = True) -> float:
    return _lib.load().ermod_getscrn(float(ewtoler), float(elecut), 1 if distance_form else 0)


def enginit_species(hist: dict, large: int = 10000):
    h = np.array([hist[k] for k in ("ecdmin", "ecfmns", "ecdcen", "eccore", "ecdmax",
                                    "eclbin", "ecfbin", "ec0bin", "finfac")], dtype=np.float64)
    out = np.zeros(large)
    pemax, pesoft = C.c_int(0), C.c_int(0)
    _lib.check(_lib.load().ermod_enginit_species(_lib.dp(h), int(hist["pecore"]), large, _lib.dp(out),
                                                 C.byref(pemax), C.byref(pesoft)), "enginit")
    return out[:pemax.value].copy(), pemax.value, pesoft.value


def enginit_bins(numslv: int, hist: dict = None):
    """One &hist for the solute self energy (pti = 0) and every solvent species."""
    hist = dict(HIST_DEFAULT if hist is None else hist)
    uvcrd, uvmax, uvsoft, escrd = [], [], [], None
    for pti in range(numslv + 1):
        crd, pemax, pesoft = enginit_species(hist)
        if pti == 0:
            escrd = crd[:pesoft].copy()
        else:
            uvcrd.append(crd)
            uvmax.append(pemax)
            uvsoft.append(pesoft)
    return dict(uvcrd=np.concatenate(uvcrd), uvmax=np.array(uvmax, np.int32),
                uvsoft=np.array(uvsoft, np.int32), escrd=escrd, esmax=len(escrd))


def setparam_topology(species, slttype: int, ljformat: int = 0, cmbrule: int = 0):
    """species: list of dicts {count, sluvid, charge, eps, len} in MDinfo order."""
    eps_all = np.concatenate([np.asarray(sp["eps"], np.float64) for sp in species])
    len_all = np.concatenate([np.asarray(sp["len"], np.float64) for sp in species])
    n = len(eps_all)
    ljt = np.zeros(n, np.int32)
    tmax = C.c_int(0)
    ljene = np.zeros(n * n)
    ljlensq = np.zeros(n * n)
    _lib.check(_lib.load().ermod_lj_tables(n, _lib.dp(eps_all), _lib.dp(len_all), ljformat, cmbrule, n,
                                           _lib.ip(ljt), C.byref(tmax), _lib.dp(ljene), _lib.dp(ljlensq)),
               "lj_tables")
    T = tmax.value
    ljene = ljene[:T * T].reshape(T, T, order="F")
    ljlensq = ljlensq[:T * T].reshape(T, T, order="F")
    ljtype, charge, mbi, sluvid, moltype = [], [], [1], [], []
    off = 0
    for t, sp in enumerate(species, start=1):
        q = np.asarray(sp["charge"], np.float64)
        types = ljt[off:off + len(q)]
        off += len(q)
        for _ in range(sp["count"]):
            ljtype.extend(types.tolist())
            charge.extend(q.tolist())
            mbi.append(mbi[-1] + len(q))
            sluvid.append(sp["sluvid"])
            moltype.append(t)
    charge = CHARGE_SCALE * np.array(charge, np.float64)
    mbi = np.array(mbi, np.int32)
    nummol = len(sluvid)
    sluvid = np.array(sluvid, np.int32)
    moltype = np.array(moltype, np.int32)
    numslt = int(np.count_nonzero(sluvid > 0))
    solute_moltype = int(moltype[sluvid > 0][-1])
    numslv = len(species) - 1 if numslt == 1 else len(species)
    uvspec = moltype.copy()
    if numslt == 1:
        uvspec[sluvid != 0] = 0
        uvspec[(sluvid == 0) & (moltype > solute_moltype)] -= 1
    return dict(nummol=nummol, numatm=int(mbi[-1] - 1), mol_begin_index=mbi, sluvid=sluvid,
                uvspec=uvspec.astype(np.int32), moltype=moltype, charge=charge,
                ljtype=np.array(ljtype, np.int32), ljtype_max=T,
                ljene_mat=np.asfortranarray(ljene), ljlensq_mat=np.asfortranarray(ljlensq),
                numslv=numslv, numslt=numslt)
