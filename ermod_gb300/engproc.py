"""Host-side front end of the GB300 path, shaped like ERmod's engproc module.

``EnergyRepresentation`` holds one ``ermod_ctx`` and exposes the reference's per-frame
protocol (engproc.F90): ``engclear`` (:276-288), ``engconst`` = ``frame`` (:355-383)
+ ``placements`` (:388-392), and the accumulators that ``engstore`` (:451-659) turns
into engsln/engref/corref.  Every call goes through the C ABI of
``libermod_gb300.so``; a nonzero status raises ``ErmodError`` whose ``name`` is the
reference's ``halt_with_error`` identity (``eng_min``, ``eng_sft``, ...).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import ErmodError, check  # noqa: F401

PARAM_KEYS = ("slttype", "estype", "ljswitch", "splodr", "ms1max", "ms2max", "ms3max", "wgtslf", "corrcal",
              "selfcal", "force_calculation", "elecut", "lwljcut", "upljcut", "screen", "temp",
              "block_threshold", "boxshp")


class EnergyRepresentation:
    def __init__(self, params: dict, topo: dict, bins: dict, precision: str = "mixed", device: int = 0,
                 batch: int = 0, count_mirror: bool = False, finish_group: int = 0):
        L = _lib.load()
        p = _lib.Params()
        L.ermod_default_params(C.byref(p))
        for k in PARAM_KEYS:
            if k in params:
                setattr(p, k, params[k])
        p.cltype = int(params.get("cltype", 2))  # 2 PME, 3 PPPM
        p.precision = _lib.PRECISION_MIXED if precision == "mixed" else _lib.PRECISION_FP64
        p.batch = int(batch)
        p.count_mirror = 1 if count_mirror else 0
        p.finish_group = int(finish_group)
        self.params = dict(params)
        self.precision = precision
        self.device = int(device)
        self.ctx = C.c_void_p()
        check(L.ermod_create(C.byref(p), int(device), C.byref(self.ctx)), "ermod_create")
        self.set_topology(topo)
        self.set_bins(bins)

    # -------------------------------------------------------------------------
    def close(self):
        if self.ctx:
            _lib.load().ermod_destroy(self.ctx)
            self.ctx = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_topology(self, topo: dict):
        L = _lib.load()
        self._keep = dict(
            mbi=np.ascontiguousarray(topo["mol_begin_index"], np.int32),
            sluvid=np.ascontiguousarray(topo["sluvid"], np.int32),
            uvspec=np.ascontiguousarray(topo["uvspec"], np.int32),
            charge=np.ascontiguousarray(topo["charge"], np.float64),
            ljtype=np.ascontiguousarray(topo["ljtype"], np.int32),
            ljene=np.asfortranarray(topo["ljene_mat"], np.float64).ravel(order="F").copy(),
            ljlensq=np.asfortranarray(topo["ljlensq_mat"], np.float64).ravel(order="F").copy())
        k = self._keep
        check(L.ermod_set_topology(self.ctx, int(topo["nummol"]), int(topo["numatm"]), _lib.ip(k["mbi"]),
                                   _lib.ip(k["sluvid"]), _lib.ip(k["uvspec"]), _lib.dp(k["charge"]),
                                   _lib.ip(k["ljtype"]), int(topo["ljtype_max"]), _lib.dp(k["ljene"]),
                                   _lib.dp(k["ljlensq"])), "ermod_set_topology")
        self.topo = topo

    def set_bins(self, bins: dict):
        L = _lib.load()
        uvmax = np.ascontiguousarray(bins["uvmax"], np.int32)
        uvsoft = np.ascontiguousarray(bins["uvsoft"], np.int32)
        uvcrd = np.ascontiguousarray(bins["uvcrd"], np.float64)
        escrd = np.ascontiguousarray(bins["escrd"], np.float64)
        check(L.ermod_set_bins(self.ctx, len(uvmax), _lib.ip(uvmax), _lib.ip(uvsoft), _lib.dp(uvcrd),
                               int(bins["esmax"]), _lib.dp(escrd)), "ermod_set_bins")
        self.bins = bins
        s = self.sizes()
        self.slvmax, self.ermax, self.esmax, self.numslv = s

    def set_aggregate(self, host_mol, sitemass):
        """The host aggregate (hostspec, com_aggregate insertion.F90:539-566): host_mol[i] != 0
        for the 0-based molecules i that form it; sitemass holds one mass per site."""
        hm = np.ascontiguousarray(host_mol, np.int32)
        sm = np.ascontiguousarray(sitemass, np.float64)
        if len(hm) != int(self.topo["nummol"]) or len(sm) != int(self.topo["numatm"]):
            raise ValueError("host_mol needs one entry per molecule and sitemass one per site")
        self._agg_keep = (hm, sm)
        check(_lib.load().ermod_set_aggregate(self.ctx, _lib.ip(hm), _lib.dp(sm)), "ermod_set_aggregate")

    def set_reference_structure(self, ref_mol, refhost_crd, refhost_weight, refslt_crd, refslt_weight):
        """The reference structure (load_refstructure, insertion.F90:619-700): the refspec
        molecules (ref_mol[i] != 0) whose atoms in order have reference coordinates
        refhost_crd (n, 3) and weights refhost_weight (n), and the solute's refslt_crd (ns, 3)
        and refslt_weight (ns)."""
        rm = np.ascontiguousarray(ref_mol, np.int32)
        hc = np.ascontiguousarray(refhost_crd, np.float64).reshape(-1, 3)
        hw = np.ascontiguousarray(refhost_weight, np.float64)
        sc = np.ascontiguousarray(refslt_crd, np.float64).reshape(-1, 3)
        sw = np.ascontiguousarray(refslt_weight, np.float64)
        if len(rm) != int(self.topo["nummol"]) or len(hc) != len(hw) or len(sc) != len(sw):
            raise ValueError("ref_mol needs one entry per molecule; coordinates and weights must pair up")
        self._ref_keep = (rm, hc, hw, sc, sw)
        check(_lib.load().ermod_set_reference_structure(self.ctx, _lib.ip(rm), _lib.dp(hc), _lib.dp(hw), len(sc),
                                                        _lib.dp(sc), _lib.dp(sw)), "ermod_set_reference_structure")

    def set_solute_library(self, conf, weight=None, insstructure: int = 0, lwstr: float = 0.0,
                           upstr: float = 0.0):
        """A flexible solute (slttype 3, getsolute in insertion.F90:384-495): SltConf's
        structures conf (nconf, nsite, 3) in file order and SltWght's weights (or None); with
        insstructure 1 only structures whose best-fit RMSD from the reference solute lies in
        [lwstr, upstr] are used.  generate_placements then takes placement g's structure and
        initial weight from the g-th accepted read of the wrapped files.  conf None removes
        the library."""
        if conf is None:
            check(_lib.load().ermod_set_solute_library(self.ctx, 0, 0, None, 0, None, 0, 0.0, 0.0),
                  "ermod_set_solute_library")
            return
        cf = np.ascontiguousarray(conf, np.float64)
        if cf.ndim != 3 or cf.shape[2] != 3:
            raise ValueError("conf must be (nconf, nsite, 3)")
        wt = None if weight is None else np.ascontiguousarray(weight, np.float64)
        check(_lib.load().ermod_set_solute_library(self.ctx, cf.shape[0], cf.shape[1], _lib.dp(cf),
                                                   0 if wt is None else len(wt), _lib.dp(wt), int(insstructure),
                                                   float(lwstr), float(upstr)), "ermod_set_solute_library")

    def set_configuration_check(self, insposition: int, lwreg: float = 0.0, upreg: float = 0.0,
                                insstructure: int = 0, lwstr: float = 0.0, upstr: float = 0.0):
        """check_mol_configuration (engproc.F90:1046-1100) for solution mode: a placement whose
        solute fails the position test (insposition 2 sphere, 3 slab, 4 symmetric slab about
        the host aggregate; 5 RMSD from the reference solute carried into the frame by the host
        fit) or the structure test (insstructure 1: best-fit RMSD in [lwstr, upstr]) is
        skipped; 0, 1 and 6 test no position."""
        check(_lib.load().ermod_set_configuration_check(self.ctx, int(insposition), float(lwreg), float(upreg),
                                                        int(insstructure), float(lwstr), float(upstr)),
              "ermod_set_configuration_check")

    def sizes(self):
        a, b, c, d = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        check(_lib.load().ermod_get_sizes(self.ctx, C.byref(a), C.byref(b), C.byref(c), C.byref(d)), "sizes")
        return a.value, b.value, c.value, d.value

    # ---- engconst --------------------------------------------------------------
    def frame(self, sitepos: np.ndarray, cell: np.ndarray, stat_weight_system: float = 1.0):
        sp = np.ascontiguousarray(sitepos, np.float64)
        cl = np.asfortranarray(cell, np.float64).ravel(order="F").copy()
        check(_lib.load().ermod_frame(self.ctx, _lib.dp(sp), _lib.dp(cl), float(stat_weight_system)),
              "ermod_frame")

    def placements(self, tagslt, solute_sitepos=None, stat_weight_solute=None, want_uvengy=False,
                   want_flceng=False):
        tag = np.ascontiguousarray(np.atleast_1d(tagslt), np.int32)
        n = len(tag)
        sx = None if solute_sitepos is None else np.ascontiguousarray(solute_sitepos, np.float64)
        sw = None if stat_weight_solute is None else np.ascontiguousarray(stat_weight_solute, np.float64)
        uv = np.zeros((n, self.slvmax + 1)) if want_uvengy else None
        fl = np.zeros((n, self.numslv)) if want_flceng else None
        check(_lib.load().ermod_placements(self.ctx, n, _lib.ip(tag), _lib.dp(sx), _lib.dp(sw), _lib.dp(uv),
                                           _lib.dp(fl)), "ermod_placements")
        return dict(uvengy=uv, flceng=fl)

    def engconst(self, sitepos, cell, tagslt, solute_sitepos=None, stat_weight_system=1.0, **kw):
        self.frame(sitepos, cell, stat_weight_system)
        return self.placements(tagslt, solute_sitepos, **kw)

    def engclear(self):
        check(_lib.load().ermod_clear(self.ctx), "ermod_clear")

    def accum(self, with_count: bool = False):
        E, S, N = self.ermax, self.esmax, self.numslv
        edens = np.zeros(E)
        ecorr = np.zeros(E * E) if self.params.get("corrcal") else None
        cnt = np.zeros(E * E, np.int64) if with_count else None
        eself = np.zeros(max(S, 1))
        slnuv = np.zeros(N)
        mn, mx = np.zeros(N + 1), np.zeros(N + 1)
        sc = np.zeros(5)
        check(_lib.load().ermod_get_accum(self.ctx, _lib.dp(edens), _lib.dp(ecorr), _lib.dp(eself), _lib.dp(slnuv),
                                          _lib.dp(mn), _lib.dp(mx), _lib.dp(sc), _lib.i64p(cnt)), "ermod_get_accum")
        return dict(edens=edens, ecorr=None if ecorr is None else ecorr.reshape(E, E, order="F"),
                    ecorr_count=None if cnt is None else cnt.reshape(E, E, order="F"), eself=eself[:S],
                    slnuv=slnuv, minuv=mn, maxuv=mx, engnorm=sc[0], engsmpl=sc[1], avslf=sc[2], voffset=sc[3],
                    voffset_initialized=bool(sc[4]))

    # ---- placements generated on the device ----------------------------------------
    def generate_placements(self, n: int, bfcoord, mass, insposition: int = 0, insorient: int = 0,
                            insorigin: int = 0, lwreg: float = 0.0, upreg: float = 0.0, seed: int = 1,
                            offset: int = 0, weights: bool = False):
        """n placements of a solute with reference coordinates bfcoord (nsite, 3) and masses,
        generated on the device in the cell of the last frame (insertion.F90 modes;
        insorigin 2 needs set_aggregate, 3 set_reference_structure; with a structure library
        (set_solute_library) bfcoord is not used and may be None).  Returns torch tensors
        (placements (n, nsite, 3) float64, weights (n,) or None); a placement the RMSD
        acceptance of insorigin 3 cannot place raises ErmodError ('ins_geo')."""
        import torch
        bf = None if bfcoord is None else np.ascontiguousarray(bfcoord, np.float64)
        m = np.ascontiguousarray(mass, np.float64)
        ns = len(m)
        dev = torch.device("cuda", self.device)
        sol = torch.empty((n, ns, 3), dtype=torch.float64, device=dev)
        sws = torch.empty(n, dtype=torch.float64, device=dev) if weights else None
        torch.cuda.synchronize(dev)
        ip = _lib.InsertParams(int(insposition), int(insorient), int(insorigin), 0, float(lwreg), float(upreg),
                               int(seed), int(offset))
        check(_lib.load().ermod_generate_placements(self.ctx, int(n), ns, _lib.dp(bf), _lib.dp(m), C.byref(ip),
                                                    C.c_void_p(sol.data_ptr()),
                                                    C.c_void_p(sws.data_ptr()) if weights else None),
              "ermod_generate_placements")
        check(_lib.load().ermod_sync(self.ctx), "ermod_generate_placements")
        return sol, sws

    def sync_stream(self):
        """Wait for the context's stream (no status decode)."""
        import torch
        torch.cuda.synchronize(torch.device("cuda", self.device))

    # ---- intermediate-state extension ------------------------------------------------
    def intermediate_enable(self, refs_density):
        """Solution mode: the zero-density bins of the reference-solvent distribution."""
        check(_lib.load().ermod_intermediate_enable(self.ctx, _lib.dp(np.ascontiguousarray(refs_density,
                                                                                          np.float64))),
              "ermod_intermediate_enable")

    def intermediate_get(self):
        ed, uv, tot = np.zeros(self.ermax), np.zeros(self.numslv), np.zeros(3)
        check(_lib.load().ermod_intermediate_get(self.ctx, _lib.dp(ed), _lib.dp(uv), _lib.dp(tot)),
              "ermod_intermediate_get")
        return dict(edintm=ed, uvintm=uv, soln_total=tot[0], soln_intm=tot[1], norm_intm=tot[2])

    # ---- adjoint mode ------------------------------------------------------------
    def adjoint_enable(self, solute_mol: int = None, cmbrule: int = 0):
        """Accumulate bin-resolved d u / d(q_s, eps_s, sigma_s) for placements of solute_mol
        (1-based; default the last molecule, the solute of an MDinfo-ordered topology)."""
        mol = self.topo["nummol"] if solute_mol is None else int(solute_mol)
        check(_lib.load().ermod_adjoint_enable(self.ctx, mol, int(cmbrule)), "ermod_adjoint_enable")
        ns = int(self.topo["mol_begin_index"][mol] - self.topo["mol_begin_index"][mol - 1])
        self._adj_nparam = 3 * ns

    def adjoint_get(self):
        """(grad [3 nsite, ermax], weight [ermax]); <du/dtheta_p> in bin i is grad[p, i] / weight[i]."""
        P = self._adj_nparam
        grad = np.zeros(P * self.ermax)
        w = np.zeros(self.ermax)
        n = C.c_int()
        check(_lib.load().ermod_adjoint_get(self.ctx, _lib.dp(grad), _lib.dp(w), C.byref(n)), "ermod_adjoint_get")
        return grad.reshape(P, self.ermax), w

    def error_info(self):
        p, m, e = C.c_int(), C.c_int(), C.c_double()
        check(_lib.load().ermod_error_info(self.ctx, C.byref(p), C.byref(m), C.byref(e)), "error_info")
        return p.value, m.value, e.value

    # ---- instrumentation ---------------------------------------------------------
    def timing(self, on: bool = True):
        check(_lib.load().ermod_timing_enable(self.ctx, 1 if on else 0), "timing")

    def timing_reset(self):
        check(_lib.load().ermod_timing_reset(self.ctx), "timing_reset")

    def timing_get(self):
        ms = (C.c_double * 16)()
        names = (C.c_char_p * 16)()
        n = C.c_int()
        launches = C.c_int64()
        check(_lib.load().ermod_timing_get(self.ctx, 16, ms, names, C.byref(n), C.byref(launches)), "timing_get")
        return {names[i].decode(): ms[i] for i in range(n.value)}, launches.value

    def set_stream(self, stream_handle: int):
        check(_lib.load().ermod_set_stream(self.ctx, C.c_void_p(stream_handle)), "set_stream")

    # ---- device-resident inputs (pointers as ints) ----------------------------------
    def frame_device(self, sitepos_ptr: int, cell, stat_weight_system: float = 1.0):
        cl = np.asfortranarray(cell, np.float64).ravel(order="F").copy()
        check(_lib.load().ermod_frame_device(self.ctx, C.c_void_p(sitepos_ptr), _lib.dp(cl),
                                             float(stat_weight_system)), "ermod_frame_device")

    def placements_device(self, n: int, tag_ptr: int, sol_ptr: int = 0, sws_ptr: int = 0):
        check(_lib.load().ermod_placements_device(self.ctx, int(n), C.c_void_p(tag_ptr),
                                                  C.c_void_p(sol_ptr or None), C.c_void_p(sws_ptr or None),
                                                  None, None), "ermod_placements_device")

    def sync(self):
        check(_lib.load().ermod_sync(self.ctx), "ermod_sync")
