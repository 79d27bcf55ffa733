"""engstore: merge of per-rank accumulators and normalisation (engproc.F90:451-560).

ERmod shards frames over MPI ranks (plmode = 2) and reduces the accumulators in
``engstore``: MAX of ``voffset`` with a per-rank rescale exp(+-(voffset_local -
voffset)/kT), SUM of engnorm/engsmpl/avslf/eself/slnuv/edens/ecorr, MIN/MAX of
minuv/maxuv, then division by engnorm.  Here every GPU (one process per GPU) owns a
shard of the frames; the exchange is the same reduction, done on the host through
``ermod_engstore_merge`` after gathering the raw accumulators with
``torch.distributed`` (any backend: NCCL between GPU ranks, gloo on CPU).
"""
from __future__ import annotations

import numpy as np

from . import _lib


def merge(accums: list, slttype: int, wgtslf: int, temp: float) -> dict:
    """accums: raw accumulators (EnergyRepresentation.accum() dicts) of every rank."""
    n = len(accums)
    E = len(accums[0]["edens"])
    S = len(accums[0]["eself"])
    N = len(accums[0]["slnuv"])
    has_corr = accums[0].get("ecorr") is not None
    edens = np.ascontiguousarray(np.stack([a["edens"] for a in accums]), np.float64)
    ecorr = (np.ascontiguousarray(np.stack([np.asarray(a["ecorr"]).ravel(order="F") for a in accums]), np.float64)
             if has_corr else None)
    eself = np.ascontiguousarray(np.stack([a["eself"] for a in accums]), np.float64) if S else None
    slnuv = np.ascontiguousarray(np.stack([a["slnuv"] for a in accums]), np.float64)
    minuv = np.ascontiguousarray(np.stack([a["minuv"] for a in accums]), np.float64)
    maxuv = np.ascontiguousarray(np.stack([a["maxuv"] for a in accums]), np.float64)
    sc = np.ascontiguousarray(np.stack([[a["engnorm"], a["engsmpl"], a["avslf"], a["voffset"],
                                         1.0 if a["voffset_initialized"] else 0.0] for a in accums]), np.float64)
    _lib.check(_lib.load().ermod_engstore_merge(n, int(slttype), int(wgtslf), float(temp), E, S, N, _lib.dp(edens),
                                                _lib.dp(ecorr), _lib.dp(eself), _lib.dp(slnuv), _lib.dp(minuv),
                                                _lib.dp(maxuv), _lib.dp(sc)), "ermod_engstore_merge")
    return dict(edens=edens[0], ecorr=None if ecorr is None else ecorr[0].reshape(E, E, order="F"),
                eself=eself[0] if S else eself, slnuv=slnuv[0], minuv=minuv[0], maxuv=maxuv[0],
                engnorm=sc[0, 0], engsmpl=sc[0, 1], avslf=sc[0, 2], voffset=sc[0, 3])


def merge_distributed(acc: dict, slttype: int, wgtslf: int, temp: float, group=None):
    """Gather every rank's raw accumulators to rank 0 and merge there (None elsewhere)."""
    import torch.distributed as dist
    world = dist.get_world_size(group)
    rank = dist.get_rank(group)
    gathered = [None] * world if rank == 0 else None
    payload = {k: (np.asarray(v) if isinstance(v, np.ndarray) else v) for k, v in acc.items()}
    dist.gather_object(payload, gathered, dst=0, group=group)
    if rank != 0:
        return None
    return merge(gathered, slttype, wgtslf, temp)


def write_outputs(directory: str, merged: dict, bins: dict, slttype: int, corrcal: int, selfcal: int,
                  suffix: str = ".tt") -> list:
    """engstore's files from merged accumulators (engproc.F90:594-657): engsln/engref,
    corsln/corref (corrcal), slfeng (selfcal), uvrange.tt.  Returns the paths written."""
    import os
    L = _lib.load()
    soln = int(slttype) == 1
    paths = []

    def path(name):
        p = os.path.join(directory, name)
        paths.append(p)
        return p.encode()

    uvmax = np.ascontiguousarray(bins["uvmax"], np.int32)
    uvsoft = np.ascontiguousarray(bins["uvsoft"], np.int32)
    uvcrd = np.ascontiguousarray(bins["uvcrd"], np.float64)
    edens = np.ascontiguousarray(merged["edens"], np.float64)
    _lib.check(L.ermod_write_engdist(path(("engsln" if soln else "engref") + suffix), len(uvmax), _lib.ip(uvmax),
                                     _lib.ip(uvsoft), _lib.dp(uvcrd), _lib.dp(edens)), "ermod_write_engdist")
    if corrcal and merged.get("ecorr") is not None:
        ec = np.asfortranarray(merged["ecorr"], np.float64).ravel(order="F").copy()
        _lib.check(L.ermod_write_corr(path(("corsln" if soln else "corref") + suffix), len(edens), _lib.dp(ec)),
                   "ermod_write_corr")
    if selfcal and merged.get("eself") is not None and len(merged["eself"]):
        es = np.ascontiguousarray(merged["eself"], np.float64)
        escrd = np.ascontiguousarray(bins["escrd"], np.float64)
        _lib.check(L.ermod_write_selfdist(path("slfeng" + suffix), len(es), _lib.dp(escrd), _lib.dp(es)),
                   "ermod_write_selfdist")
    mn = np.ascontiguousarray(merged["minuv"], np.float64)
    mx = np.ascontiguousarray(merged["maxuv"], np.float64)
    _lib.check(L.ermod_write_uvrange(path("uvrange.tt"), len(mn) - 1, _lib.dp(mn), _lib.dp(mx)),
               "ermod_write_uvrange")
    return paths


def format_g(x: float, w: int, d: int) -> str:
    """The Fortran Gw.d field the writers produce."""
    import ctypes as C
    buf = C.create_string_buffer(w + 8)
    _lib.check(_lib.load().ermod_format_g(float(x), int(w), int(d), buf, w + 8), "ermod_format_g")
    return buf.value.decode()


def read_engdist(path: str) -> np.ndarray:
    """The third column (density) of an engsln/engref file, read list-directed as slvfe does."""
    return np.array([float(ln.split()[2]) for ln in open(path) if ln.strip()])


def refs_density_for_intermediate(prefix: str) -> np.ndarray:
    """The reference-solvent density the intermediate-state extension tests against:
    prefix + '.tt' when it exists, else the largest over prefix + '.01' .. '.99'
    (extensions/Intermediate/engproc.F90:286-316)."""
    import os
    if os.path.exists(prefix + ".tt"):
        return read_engdist(prefix + ".tt")
    out = None
    for k in range(1, 100):
        p = f"{prefix}.{k:02d}"
        if os.path.exists(p):
            d = read_engdist(p)
            out = d if out is None else np.maximum(out, d)
    if out is None:
        raise FileNotFoundError(prefix)
    return out


def write_intermediate(directory: str, intm: dict, bins: dict, temp: float, division: int, engdiv: int,
                       avintm_rows: list = None) -> list:
    """The extension's outputs: engint.xx (edintm / norm_intm in engsln's layout), and at
    the last division Prob_Result and avint.tt (extensions/Intermediate/engproc.F90:623-693).
    avintm_rows: uvintm / norm_intm of every division so far (for avint.tt)."""
    import os
    L = _lib.load()
    suffix = ".tt" if engdiv == 1 else f".{division:02d}"
    paths = []
    uvmax = np.ascontiguousarray(bins["uvmax"], np.int32)
    uvsoft = np.ascontiguousarray(bins["uvsoft"], np.int32)
    uvcrd = np.ascontiguousarray(bins["uvcrd"], np.float64)
    ed = np.ascontiguousarray(intm["edintm"] / intm["norm_intm"], np.float64)
    p = os.path.join(directory, "engint" + suffix)
    _lib.check(L.ermod_write_engdist(p.encode(), len(uvmax), _lib.ip(uvmax), _lib.ip(uvsoft), _lib.dp(uvcrd),
                                     _lib.dp(ed)), "ermod_write_engdist")
    paths.append(p)
    if division == engdiv:
        factor = intm["soln_intm"] / intm["soln_total"]
        p = os.path.join(directory, "Prob_Result")
        with open(p, "w") as f:
            f.write(" Probability to find the system in the intermediate state = %12.6f\n" % factor)
            f.write(" Free-energy change from the intermediate state to the simulated state\n")
            f.write("                                                = %12.6f kcal/mol\n" % (temp * np.log(factor)))
        paths.append(p)
        rows = avintm_rows if avintm_rows is not None else [intm["uvintm"] / intm["norm_intm"]]
        p = os.path.join(directory, "avint.tt")
        with open(p, "w") as f:
            for k, row in enumerate(rows, start=1):  # format(i5, 9999f15.5)
                f.write("%5d" % k + "".join("%15.5f" % v for v in row) + "\n")
        paths.append(p)
    return paths
