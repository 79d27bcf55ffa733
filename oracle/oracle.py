"""Python front end of the FP64 CPU oracle.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and the
``cpu_baseline`` / ``--impl reference`` legs of ``bench.py`` may import this module,
and only as the checker or the timed CPU restatement of the reference.

Parity status: partially pinned -- see ``oracle/ermod_oracle.h``.

Contents
  * ctypes binding of ``oracle/build/liboracle.so`` (built by ``oracle/Makefile``),
  * ``setparam_topology``: a numpy restatement of the set-up semantics of
    ``setconf.F90:720-834`` (LJ-type deduplication, combination rules, charge
    scaling, molecular charges) and of the species numbering of
    ``engproc.F90:102-120`` (``uvspec``),
  * ``enginit_bins``: the energy-coordinate construction of ``engproc.F90:122-237``,
  * ``Oracle``: the per-frame engine (``engconst`` / ``update_histogram``).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "build", "liboracle.so")

CHARGE_SCALE = 18.22261721          # setconf.F90:829
SGMCNV = 1.7817974362806784         # setconf.F90:566, Rmin/2 -> sigma
LENCNV = 10.0                       # nm -> Angstrom
ENGCNV = 1.0 / 4.184                # kJ/mol -> kcal/mol

OK = 0
E_ENG_MIN, E_ENG_SFT, E_ENG_BUG, E_ENG_CNS, E_RCP_CNS, E_RCP_FST = 101, 102, 103, 104, 105, 106
W_MBIN, E_PARAM, E_NONCUBOID = 110, 120, 121
E_ENG_SLB = 109


class OrcParams(C.Structure):
    _fields_ = [
        ("slttype", C.c_int32), ("estype", C.c_int32), ("ljswitch", C.c_int32),
        ("splodr", C.c_int32), ("ms1max", C.c_int32), ("ms2max", C.c_int32),
        ("ms3max", C.c_int32), ("wgtslf", C.c_int32), ("corrcal", C.c_int32),
        ("selfcal", C.c_int32), ("force_calculation", C.c_int32), ("elmode", C.c_int32),
        ("elecut", C.c_double), ("lwljcut", C.c_double), ("upljcut", C.c_double),
        ("screen", C.c_double), ("temp", C.c_double), ("block_threshold", C.c_double),
        ("boxshp", C.c_int32), ("reserved_", C.c_int32),
    ]


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (g++, OpenMP)."""
    src = os.path.join(HERE, "ermod_oracle.cpp")
    if force or not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < max(
            os.path.getmtime(src), os.path.getmtime(os.path.join(HERE, "ermod_oracle.h"))):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        dp, ip = C.POINTER(C.c_double), C.POINTER(C.c_int)
        L.orc_spline_value.restype = C.c_double
        L.orc_spline_value.argtypes = [C.c_int, C.c_double]
        L.orc_getscrn.restype = C.c_double
        L.orc_getscrn.argtypes = [C.c_double, C.c_double, C.c_int]
        L.orc_enginit_species.argtypes = [dp, C.c_int, C.c_int, dp, ip, ip]
        L.orc_fft_r2c_3d.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp]
        L.orc_fft_c2r_3d.argtypes = [C.c_int, C.c_int, C.c_int, dp, dp]
        L.orc_pair_energy.restype = C.c_double
        L.orc_pair_energy.argtypes = [C.POINTER(OrcParams), C.c_double, C.c_double, C.c_double, C.c_double]
        L.orc_create.argtypes = [C.POINTER(OrcParams), C.POINTER(C.c_void_p)]
        L.orc_destroy.argtypes = [C.c_void_p]
        L.orc_destroy.restype = None
        L.orc_set_topology.argtypes = [C.c_void_p, C.c_int, C.c_int, ip, ip, ip, dp, ip, C.c_int, dp, dp]
        L.orc_set_bins.argtypes = [C.c_void_p, C.c_int, ip, ip, dp, C.c_int, dp]
        L.orc_frame.argtypes = [C.c_void_p, dp, dp, C.c_double]
        L.orc_placements.argtypes = [C.c_void_p, C.c_int, ip, dp, dp, dp, dp, C.c_int]
        L.orc_slvmax.argtypes = [C.c_void_p]
        L.orc_clear.argtypes = [C.c_void_p]
        L.orc_get_accum.argtypes = [C.c_void_p, dp, dp, dp, dp, dp, dp, dp]
        L.orc_last_cnvslt.argtypes = [C.c_void_p, dp, dp]
        L.orc_direct_ewald.argtypes = [C.c_void_p, C.c_int, dp, C.c_int, dp, dp]
        L.orc_recip_parts.argtypes = [C.c_void_p, C.c_int, dp, dp, dp]
        L.orc_adjoint.argtypes = [C.c_void_p, C.c_int, dp, C.c_int, dp]
        L.orc_intermediate_enable.argtypes = [C.c_void_p, dp]
        L.orc_intermediate_get.argtypes = [C.c_void_p, dp, dp, dp]
        L.orc_set_configuration_check.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_double, C.c_int,
                                                  C.c_double, C.c_double]
        L.orc_set_aggregate.argtypes = [C.c_void_p, ip, dp]
        L.orc_set_reference_structure.argtypes = [C.c_void_p, ip, dp, dp, C.c_int, dp, dp]
        L.orc_fit_a_rotate_b.argtypes = [C.c_int, dp, dp, dp, C.c_int, dp, dp]
        _lib = L
    return _lib


def _dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def _ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


class OracleError(RuntimeError):
    def __init__(self, code, where):
        super().__init__(f"oracle {where}: status {code}")
        self.code = code


def _check(code, where):
    if code != OK:
        raise OracleError(code, where)


# ----------------------------------------------------------------------------------
# routines with golden vectors / analytic checks
# ----------------------------------------------------------------------------------
def fit_a_rotate_b(refa, a, massa, b):
    """bestfit.F90 fit_a_rotate_b: a (na, 3) fitted onto refa with weights massa; returns b
    (nb, 3) under the same transform."""
    refa = np.ascontiguousarray(refa, np.float64)
    a = np.ascontiguousarray(a, np.float64)
    m = np.ascontiguousarray(massa, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    out = np.zeros_like(b)
    _check(lib().orc_fit_a_rotate_b(len(a), _dp(refa), _dp(a), _dp(m), len(b), _dp(b), _dp(out)), "fit_a_rotate_b")
    return out


def spline_value(order: int, x: float) -> float:
    """spline.F90:47-59 (M_order(x))."""
    return lib().orc_spline_value(order, x)


def getscrn(ewtoler: float, elecut: float, dis: bool = True) -> float:
    """setconf.F90:515-535."""
    return lib().orc_getscrn(ewtoler, elecut, 1 if dis else 0)


def fft_r2c_3d(grid: np.ndarray) -> np.ndarray:
    """Reference-convention forward R2C of real[K3][K2][K1] -> complex[K3][K2][K1/2+1]."""
    g = np.ascontiguousarray(grid, dtype=np.float64)
    k3, k2, k1 = g.shape
    out = np.zeros((k3, k2, k1 // 2 + 1), dtype=np.complex128)
    _check(lib().orc_fft_r2c_3d(k1, k2, k3, _dp(g), out.ctypes.data_as(C.POINTER(C.c_double))), "fft")
    return out


def fft_c2r_3d(spec: np.ndarray, k1: int) -> np.ndarray:
    s = np.ascontiguousarray(spec, dtype=np.complex128)
    k3, k2, _ = s.shape
    out = np.zeros((k3, k2, k1), dtype=np.float64)
    _check(lib().orc_fft_c2r_3d(k1, k2, k3, s.ctypes.data_as(C.POINTER(C.c_double)), _dp(out)), "fft")
    return out


HIST_DEFAULT = dict(ecdmin=-20.0, ecfmns=-0.20, ecdcen=0.0, eccore=20.0, ecdmax=1.0e11,
                    eclbin=5.0e-2, ecfbin=2.0e-3, ec0bin=2.0e-4, finfac=10.0, pecore=200)


def enginit_species(hist: dict, large: int = 10000):
    """engproc.F90:163-218 for one species -> (ercrd[1:pemax], pemax, pesoft)."""
    h = np.array([hist[k] for k in ("ecdmin", "ecfmns", "ecdcen", "eccore", "ecdmax",
                                    "eclbin", "ecfbin", "ec0bin", "finfac")], dtype=np.float64)
    out = np.zeros(large, dtype=np.float64)
    pemax, pesoft = C.c_int(0), C.c_int(0)
    _check(lib().orc_enginit_species(_dp(h), int(hist["pecore"]), large, _dp(out),
                                     C.byref(pemax), C.byref(pesoft)), "enginit")
    return out[:pemax.value].copy(), pemax.value, pesoft.value


def enginit_bins(numslv: int, hist: dict = None):
    """engproc.F90:122-237 with one &hist for every species (peread = 0)."""
    hist = dict(HIST_DEFAULT if hist is None else hist)
    uvcrd, uvmax, uvsoft = [], [], []
    esc = None
    for pti in range(0, numslv + 1):
        crd, pemax, pesoft = enginit_species(hist)
        if pti == 0:
            esc = crd[:pesoft].copy()          # esmax = pesoft (engproc.F90:220-221)
        else:
            uvcrd.append(crd)
            uvmax.append(pemax)
            uvsoft.append(pesoft)
    return dict(uvcrd=np.concatenate(uvcrd), uvmax=np.array(uvmax, np.int32),
                uvsoft=np.array(uvsoft, np.int32), escrd=esc, esmax=len(esc))


# ----------------------------------------------------------------------------------
# set-up semantics (setconf.F90:720-834, engproc.F90:102-120)
# ----------------------------------------------------------------------------------
def setparam_topology(species, slttype: int, ljformat: int = 0, cmbrule: int = 0):
    """Build the engmain topology state from per-species site tables.

    ``species``: list (in MDinfo order) of dicts with keys ``count``, ``sluvid``
    (0 solvent, 1 solute, 2/3 test particle), ``charge`` (e), ``eps`` and ``len``
    (in ``ljformat`` units).  The molecule type is the species' position + 1.
    """
    lj_len_tab, lj_eps_tab = [], []
    ljtype, charge, mbi, sluvid, moltype = [], [], [1], [], []
    for t, sp in enumerate(species, start=1):
        q = np.asarray(sp["charge"], np.float64)
        e = np.asarray(sp["eps"], np.float64).copy()
        ln = np.asarray(sp["len"], np.float64).copy()
        if ljformat == 1:
            ln = SGMCNV * ln
        if ljformat in (3, 4):
            for s in range(len(e)):
                if ln[s] != 0.0:
                    factor = (e[s] / ln[s]) ** (1.0 / 6.0)
                    e[s] = ln[s] / (4.0 * (factor ** 6))
                    ln[s] = factor
                else:
                    e[s] = 0.0
        if ljformat in (2, 4):
            e = ENGCNV * e
            ln = LENCNV * ln
        types = []
        for s in range(len(q)):            # linear search of the LJ table (setconf.F90:755-775)
            found = None
            for i, (l0, e0) in enumerate(zip(lj_len_tab, lj_eps_tab)):
                if l0 == ln[s] and e0 == e[s]:
                    found = i + 1
                    break
            if found is None:
                lj_len_tab.append(ln[s])
                lj_eps_tab.append(e[s])
                found = len(lj_len_tab)
            types.append(found)
        for _ in range(sp["count"]):
            ljtype.extend(types)
            charge.extend(q.tolist())
            mbi.append(mbi[-1] + len(q))
            sluvid.append(sp["sluvid"])
            moltype.append(t)
    n = len(lj_len_tab)
    L = np.array(lj_len_tab)
    E = np.array(lj_eps_tab)
    ljlensq = np.zeros((n, n))
    ljene = np.zeros((n, n))
    for i in range(n):                       # setconf.F90:805-823 (column i)
        if cmbrule == 0:
            ljlensq[:, i] = ((L + L[i]) / 2.0) ** 2
        else:
            ljlensq[:, i] = L * L[i]
        ljene[:, i] = np.sqrt(E * E[i])
    charge = CHARGE_SCALE * np.array(charge, np.float64)
    mbi = np.array(mbi, np.int32)
    nummol = len(sluvid)
    mol_charge = np.array([charge[mbi[i] - 1:mbi[i + 1] - 1].sum() for i in range(nummol)])
    sluvid = np.array(sluvid, np.int32)
    moltype = np.array(moltype, np.int32)
    # uvspec (engproc.F90:102-120)
    numslt = int(np.count_nonzero(sluvid > 0))
    solute_moltype = int(moltype[sluvid > 0][-1])
    numtype = len(species)
    numslv = numtype - 1 if numslt == 1 else numtype
    uvspec = moltype.copy()
    if numslt == 1:
        uvspec[sluvid != 0] = 0
        uvspec[(sluvid == 0) & (moltype > solute_moltype)] -= 1
    return dict(nummol=nummol, numatm=int(mbi[-1] - 1), mol_begin_index=mbi, sluvid=sluvid,
                uvspec=uvspec.astype(np.int32), moltype=moltype, charge=charge,
                ljtype=np.array(ljtype, np.int32), ljtype_max=n,
                ljene_mat=np.asfortranarray(ljene), ljlensq_mat=np.asfortranarray(ljlensq),
                mol_charge=mol_charge, numslv=numslv, numslt=numslt)


# ----------------------------------------------------------------------------------
# the engine
# ----------------------------------------------------------------------------------
class Oracle:
    """The reference's per-frame path on the CPU (FP64), same call shape as the C-ABI."""

    def __init__(self, params: dict, topo: dict, bins: dict):
        L = lib()
        p = OrcParams()
        for name, _ in OrcParams._fields_:
            if name in params:
                setattr(p, name, params[name])
        p.elmode = {2: 0, 3: 1, 0: 2}[int(params.get("cltype", 2))]
        p.boxshp = int(params.get("boxshp", 1))
        self.params = dict(params)
        self.ctx = C.c_void_p()
        _check(L.orc_create(C.byref(p), C.byref(self.ctx)), "create")
        self.topo = topo
        self.bins = bins
        mbi = np.ascontiguousarray(topo["mol_begin_index"], np.int32)
        _check(L.orc_set_topology(self.ctx, topo["nummol"], topo["numatm"], _ip(mbi),
                                  _ip(np.ascontiguousarray(topo["sluvid"], np.int32)),
                                  _ip(np.ascontiguousarray(topo["uvspec"], np.int32)),
                                  _dp(np.ascontiguousarray(topo["charge"], np.float64)),
                                  _ip(np.ascontiguousarray(topo["ljtype"], np.int32)),
                                  topo["ljtype_max"],
                                  _dp(np.asfortranarray(topo["ljene_mat"]).ravel(order="F").copy()),
                                  _dp(np.asfortranarray(topo["ljlensq_mat"]).ravel(order="F").copy())),
               "set_topology")
        self.numslv = len(bins["uvmax"])
        self.ermax = int(np.sum(bins["uvmax"]))
        self.esmax = int(bins["esmax"])
        _check(L.orc_set_bins(self.ctx, self.numslv, _ip(np.ascontiguousarray(bins["uvmax"], np.int32)),
                              _ip(np.ascontiguousarray(bins["uvsoft"], np.int32)),
                              _dp(np.ascontiguousarray(bins["uvcrd"], np.float64)), self.esmax,
                              _dp(np.ascontiguousarray(bins["escrd"], np.float64))), "set_bins")
        self.slvmax = L.orc_slvmax(self.ctx)

    def close(self):
        if self.ctx:
            lib().orc_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def frame(self, sitepos: np.ndarray, cell: np.ndarray, stat_weight_system: float = 1.0):
        """sitepos: (numatm, 3) C-order == (3, numatm) column-major; cell: 3x3, columns = cell vectors."""
        sp = np.ascontiguousarray(sitepos, np.float64)
        cl = np.asfortranarray(cell, np.float64).ravel(order="F").copy()
        _check(lib().orc_frame(self.ctx, _dp(sp), _dp(cl), float(stat_weight_system)), "frame")

    def placements(self, tagslt, solute_sitepos=None, stat_weight_solute=None, want_uvengy=True,
                   nthreads=0, raise_on_error=True):
        tag = np.ascontiguousarray(np.atleast_1d(tagslt), np.int32)
        n = len(tag)
        sx = None if solute_sitepos is None else np.ascontiguousarray(solute_sitepos, np.float64)
        sw = None if stat_weight_solute is None else np.ascontiguousarray(stat_weight_solute, np.float64)
        uv = np.zeros((n, self.slvmax + 1)) if want_uvengy else None
        fl = np.zeros((n, self.numslv))
        st = lib().orc_placements(self.ctx, n, _ip(tag), _dp(sx), _dp(sw), _dp(uv), _dp(fl), int(nthreads))
        if raise_on_error:
            _check(st, "placements")
        return dict(status=st, uvengy=uv, flceng=fl)

    def set_aggregate(self, host_mol, sitemass):
        hm = np.ascontiguousarray(host_mol, np.int32)
        sm = np.ascontiguousarray(sitemass, np.float64)
        self._agg_keep = (hm, sm)
        _check(lib().orc_set_aggregate(self.ctx, _ip(hm), _dp(sm)), "set_aggregate")

    def set_reference_structure(self, ref_mol, refhost_crd, refhost_weight, refslt_crd, refslt_weight):
        rm = np.ascontiguousarray(ref_mol, np.int32)
        hc = np.ascontiguousarray(refhost_crd, np.float64).reshape(-1, 3)
        hw = np.ascontiguousarray(refhost_weight, np.float64)
        sc = np.ascontiguousarray(refslt_crd, np.float64).reshape(-1, 3)
        sw = np.ascontiguousarray(refslt_weight, np.float64)
        self._ref_keep = (rm, hc, hw, sc, sw)
        _check(lib().orc_set_reference_structure(self.ctx, _ip(rm), _dp(hc), _dp(hw), len(sc), _dp(sc), _dp(sw)),
               "set_reference_structure")

    def set_configuration_check(self, insposition, lwreg=0.0, upreg=0.0, insstructure=0, lwstr=0.0, upstr=0.0):
        """check_mol_configuration (engproc.F90:1046-1100), solution mode; see
        orc_set_configuration_check."""
        _check(lib().orc_set_configuration_check(self.ctx, int(insposition), float(lwreg), float(upreg),
                                                 int(insstructure), float(lwstr), float(upstr)),
               "set_configuration_check")

    def clear(self):
        _check(lib().orc_clear(self.ctx), "clear")

    def accum(self):
        E, S, N = self.ermax, self.esmax, self.numslv
        edens = np.zeros(E)
        ecorr = np.zeros(E * E) if self.params.get("corrcal") else None
        eself = np.zeros(max(S, 1))
        slnuv = np.zeros(N)
        mn, mx = np.zeros(N + 1), np.zeros(N + 1)
        sc = np.zeros(5)
        _check(lib().orc_get_accum(self.ctx, _dp(edens), _dp(ecorr), _dp(eself), _dp(slnuv), _dp(mn),
                                   _dp(mx), _dp(sc)), "get_accum")
        return dict(edens=edens, ecorr=None if ecorr is None else ecorr.reshape(E, E, order="F"),
                    eself=eself[:S], slnuv=slnuv, minuv=mn, maxuv=mx, engnorm=sc[0], engsmpl=sc[1],
                    avslf=sc[2], voffset=sc[3], voffset_initialized=bool(sc[4]))

    def last_cnvslt(self):
        K1, K2, K3 = self.params["ms1max"], self.params["ms2max"], self.params["ms3max"]
        out = np.zeros((K3, K2, K1))
        s = C.c_double(0)
        _check(lib().orc_last_cnvslt(self.ctx, _dp(out), C.byref(s)), "last_cnvslt")
        return out, s.value

    def recip_parts(self, tagslt, solute_sitepos=None):
        out = np.zeros(self.slvmax)
        s = C.c_double(0)
        sx = None if solute_sitepos is None else np.ascontiguousarray(solute_sitepos, np.float64)
        _check(lib().orc_recip_parts(self.ctx, int(tagslt), _dp(sx), _dp(out), C.byref(s)), "recip_parts")
        return out, s.value

    def direct_ewald(self, tagslt, solute_sitepos=None, mmax=12):
        out = np.zeros(self.slvmax)
        s = C.c_double(0)
        sx = None if solute_sitepos is None else np.ascontiguousarray(solute_sitepos, np.float64)
        _check(lib().orc_direct_ewald(self.ctx, int(tagslt), _dp(sx), int(mmax), _dp(out), C.byref(s)),
               "direct_ewald")
        return out, s.value

    def adjoint(self, tagslt, solute_sitepos=None, cmbrule=0):
        """(slvmax, 3 nsite) FP64 derivatives du_k / d{q_s, eps_s, sigma_s} (engine charge units)."""
        ns = int(self.topo["mol_begin_index"][tagslt] - self.topo["mol_begin_index"][tagslt - 1])
        out = np.zeros((self.slvmax, 3 * ns))
        sx = None if solute_sitepos is None else np.ascontiguousarray(solute_sitepos, np.float64)
        _check(lib().orc_adjoint(self.ctx, int(tagslt), _dp(sx), int(cmbrule), _dp(out)), "adjoint")
        return out

    def intermediate_enable(self, refs_density):
        _check(lib().orc_intermediate_enable(self.ctx, _dp(np.ascontiguousarray(refs_density, np.float64))),
               "intermediate_enable")

    def intermediate_get(self):
        ed, uv, tot = np.zeros(self.ermax), np.zeros(self.numslv), np.zeros(3)
        _check(lib().orc_intermediate_get(self.ctx, _dp(ed), _dp(uv), _dp(tot)), "intermediate_get")
        return dict(edintm=ed, uvintm=uv, soln_total=tot[0], soln_intm=tot[1], norm_intm=tot[2])
