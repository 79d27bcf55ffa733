"""GPU path vs the FP64 oracle, through the C ABI (marked gpu).

Tolerances (per molecule energy, kcal/mol):
  FP64 path   |u_gpu - u_oracle| <= 1e-9 + 1e-11 |u|
  mixed path  |u_gpu - u_oracle| <= 1e-4 + 2e-6 |u| (FP32 pair terms of overlapping
              pairs reach 1e10 kcal/mol, where only the relative error is meaningful)
Histograms: bit-exact counts except molecules whose oracle energy lies within the
observed error (at least 1e-6) of a bin edge; those are counted and reported.
"""
import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu

TOL = {"fp64": (1e-9, 1e-11), "mixed": (1e-4, 0.0)}


def _engines(gpu_lib, oracle, w, topo, bins, precision, **kw):
    from ermod_gb300.engproc import EnergyRepresentation
    gpu = EnergyRepresentation(w.params, topo, bins, precision=precision, **kw)
    orc = oracle.Oracle(w.params, topo, bins)
    return gpu, orc


def _check_energies(u_gpu, u_orc, precision):
    """Energies agree within TOL; overlapping pairs beyond 1e10 kcal/mol (above ecdmax,
    the last bin in both) only need to stay beyond it."""
    atol, rtol = TOL[precision]
    if precision == "mixed":
        rtol = 2e-6  # FP32 relative precision of large (core-region) energies
    huge = np.abs(u_orc) >= 1e10
    assert np.all(u_gpu[huge] >= 1e10)
    err = np.where(huge, 0.0, np.abs(u_gpu - u_orc))
    bound = atol + rtol * np.abs(np.where(huge, 0.0, u_orc))
    worst = int(np.argmax(err - bound))
    assert np.all(err <= bound), f"{precision}: max err {err.max():.3e} at {worst} (u={u_orc.flat[worst]:.6f})"
    soft = np.abs(u_orc) < 20.0
    return float(err[soft].max()) if np.any(soft) else 0.0


def _hist_compare(u_gpu, u_orc, edges, tol):
    """Per placement: histograms of GPU vs oracle energies agree off the bin edges."""
    flips = 0
    for ug, uo in zip(u_gpu, u_orc):
        near = helpers.near_edge(uo, edges, tol)
        hg = helpers.histogram(ug[~near], edges)
        ho = helpers.histogram(uo[~near], edges)
        assert np.array_equal(hg, ho)
        flips += int(np.count_nonzero(helpers.histogram(ug[near], edges) != helpers.histogram(uo[near], edges)))
    return flips


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_soln_small_frames(gpu_lib, oracle, precision):
    from ermod_gb300 import synth
    w = synth.soln_small()
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(gpu_lib, oracle, w, topo, bins, precision)
    tag = [topo["nummol"]]
    errs = []
    for f in range(3):
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        ro = orc.placements(tag)
        gpu.frame(pos, cell)
        rg = gpu.placements(tag, want_uvengy=True, want_flceng=True)
        errs.append(_check_energies(rg["uvengy"], ro["uvengy"], precision))
        np.testing.assert_allclose(rg["flceng"], ro["flceng"], atol=TOL[precision][0] * topo["nummol"], rtol=1e-9)
    ag, ao = gpu.accum(), orc.accum()
    edges = bins["uvcrd"]
    if precision == "fp64":
        np.testing.assert_array_equal(ag["edens"], ao["edens"])
    else:
        np.testing.assert_allclose(ag["edens"].sum(), ao["edens"].sum(), rtol=1e-12)
    for k in ("engnorm", "engsmpl", "avslf"):
        np.testing.assert_allclose(ag[k], ao[k], rtol=1e-12)
    np.testing.assert_allclose(ag["minuv"], ao["minuv"], atol=TOL[precision][0])
    np.testing.assert_allclose(ag["maxuv"], ao["maxuv"], atol=TOL[precision][0])
    # slnuv = sum of flceng * engnmfc (engnmfc = V here): the per-molecule tolerance summed
    np.testing.assert_allclose(ag["slnuv"], ao["slnuv"], rtol=0,
                               atol=3 * topo["nummol"] * TOL[precision][0] * ag["engnorm"] / 3)
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_refs_unit_weights_exact_counts(gpu_lib, oracle, precision):
    """wgtslf = 0, NVT: engnmfc = 1, so edens and ecorr are integer counts."""
    w = helpers.small_refs(wgtslf=0)
    w.params["estype"] = 1
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(gpu_lib, oracle, w, topo, bins, precision, count_mirror=True)
    pos, cell = w.frame(0)
    pl = w.placements(0, 48)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    orc.frame(pos, cell)
    ro = orc.placements(tag, pl)
    gpu.frame(pos, cell)
    rg = gpu.placements(tag, pl, want_uvengy=True)
    err = _check_energies(rg["uvengy"], ro["uvengy"], precision)
    edges = bins["uvcrd"]
    ug, uo = rg["uvengy"][:, 1:], ro["uvengy"][:, 1:]
    tol = max(1e-6, 2 * err)
    _hist_compare(ug, uo, edges, tol)
    ag, ao = gpu.accum(with_count=True), orc.accum()
    # device binning == host binning of the device's own energies
    hist_gpu = sum(helpers.histogram(u, edges) for u in ug)
    np.testing.assert_array_equal(ag["edens"], hist_gpu.astype(float))
    counts = np.zeros((len(edges), len(edges)), np.int64)
    for u in ug:
        h = helpers.histogram(u, edges).astype(np.int64)
        counts += np.outer(h, h)
    np.testing.assert_array_equal(ag["ecorr_count"], counts)
    np.testing.assert_array_equal(ag["ecorr"], counts.astype(float))
    if precision == "fp64":
        np.testing.assert_array_equal(ag["edens"], ao["edens"])
        np.testing.assert_array_equal(ag["ecorr"], ao["ecorr"])
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_refs_weighted_accumulators(gpu_lib, oracle, precision):
    """REFS defaults: wgtslf = 1, NPT; weights exp(-(u0 - voffset)/kT) V."""
    w = helpers.small_refs()
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(gpu_lib, oracle, w, topo, bins, precision, batch=16)
    for f in range(2):
        pos, cell = w.frame(f)
        pl = w.placements(f, 40)
        tag = np.full(len(pl), topo["nummol"], np.int32)
        orc.frame(pos, cell)
        ro = orc.placements(tag, pl)
        gpu.frame(pos, cell)
        rg = gpu.placements(tag, pl, want_uvengy=True)
        _check_energies(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision)
        # the solute self energy decides the weights
        np.testing.assert_allclose(rg["uvengy"][:, 0], ro["uvengy"][:, 0], atol=1e-9 if precision == "fp64" else 2e-4)
    ag, ao = gpu.accum(), orc.accum()
    rtol = 1e-10 if precision == "fp64" else 5e-4
    np.testing.assert_allclose(ag["voffset"], ao["voffset"], atol=1e-9 if precision == "fp64" else 2e-4)
    np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=rtol)
    np.testing.assert_allclose(ag["avslf"], ao["avslf"], rtol=1e-12)
    assert ag["engsmpl"] == ao["engsmpl"] == 80
    np.testing.assert_allclose(ag["edens"].sum(), ao["edens"].sum(), rtol=rtol)
    np.testing.assert_allclose(ag["ecorr"].sum(), ao["ecorr"].sum(), rtol=rtol)
    if precision == "fp64":
        np.testing.assert_allclose(ag["edens"], ao["edens"], rtol=1e-10, atol=0)
        np.testing.assert_allclose(ag["ecorr"], ao["ecorr"], rtol=1e-10, atol=0)
    gpu.close()


def test_run_to_run_deterministic(gpu_lib):
    from ermod_gb300.engproc import EnergyRepresentation
    w = helpers.small_refs()
    topo, bins = helpers.build_inputs(w)
    pos, cell = w.frame(0)
    pl = w.placements(0, 70)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    out = []
    for batch in (16, 16, 8):
        gpu = EnergyRepresentation(w.params, topo, bins, precision="mixed", batch=batch)
        gpu.frame(pos, cell)
        gpu.placements(tag, pl)
        out.append(gpu.accum())
        gpu.close()
    for k in ("edens", "ecorr", "minuv", "maxuv"):
        np.testing.assert_array_equal(out[0][k], out[1][k])
    np.testing.assert_array_equal(out[0]["edens"], out[2]["edens"])
    assert out[0]["engnorm"] == out[1]["engnorm"]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_pppm_soln_frames(gpu_lib, oracle, precision):
    """cltype 3 (PPPM): the optimal influence function replaces engfac; the rest of the path is PME's."""
    from ermod_gb300 import synth
    w = synth.soln_small()
    w.params["cltype"] = 3
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(gpu_lib, oracle, w, topo, bins, precision)
    tag = [topo["nummol"]]
    for f in range(2):
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        ro = orc.placements(tag)
        gpu.frame(pos, cell)
        rg = gpu.placements(tag, want_uvengy=True)
        _check_energies(rg["uvengy"], ro["uvengy"], precision)
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_bare_coulomb_refs_accumulators(gpu_lib, oracle, precision):
    """cltype 0: realcal_bare (LJ + q q / r within elecut), no reciprocal space, no
    residual, volcorrect without its Ewald factor."""
    w = helpers.small_refs(wgtslf=0)
    w.params["cltype"] = 0
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(gpu_lib, oracle, w, topo, bins, precision)
    pos, cell = w.frame(0)
    pl = w.placements(0, 24)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    orc.frame(pos, cell)
    ro = orc.placements(tag, pl)
    gpu.frame(pos, cell)
    rg = gpu.placements(tag, pl, want_uvengy=True)
    _check_energies(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision)
    assert np.all(rg["uvengy"][:, 0] == 0.0)
    ag, ao = gpu.accum(), orc.accum()
    np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=1e-12)
    np.testing.assert_allclose(ag["edens"].sum(), ao["edens"].sum(), rtol=1e-12)
    gpu.close()


def test_device_api_status_kept_until_sync(gpu_lib, oracle):
    """Device API: an error stays until ermod_sync reads it, later calls queued before the
    sync are stopped by it (the reference stops at its first error), and ermod_sync
    starts a new sequence.  Frame 7 of this workload stops the reference with eng_sft
    (a water jittered into the solute's core)."""
    import torch
    from ermod_gb300 import _lib, setconf, synth
    from ermod_gb300.engproc import EnergyRepresentation
    w = synth.Workload("status", "soln", 62.0, 8000, synth.random_solute(np.random.default_rng((5, 11)), 16),
                       synth._params(1, 64, corrcal=0, wgtslf=0), 5, 9, 1, 21, cavity=6.0)
    topo = setconf.setparam_topology(w.species(), slttype=1)
    bins = setconf.enginit_bins(topo["numslv"])
    orc = oracle.Oracle(w.params, topo, bins)
    st = []
    for f in (6, 7, 8):
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        st.append(orc.placements([topo["nummol"]], raise_on_error=False)["status"])
    assert st == [0, _lib.E_ENG_SFT, 0]
    dev = torch.device("cuda", 0)
    tag = torch.tensor([topo["nummol"]], dtype=torch.int32, device=dev)
    pos_d = {f: torch.from_numpy(w.frame(f)[0]).to(dev) for f in (6, 7, 8)}
    cell = w.frame(6)[1]
    eng = EnergyRepresentation(w.params, topo, bins, precision="mixed")
    torch.cuda.synchronize()
    eng.frame_device(pos_d[6].data_ptr(), cell)
    eng.placements_device(1, tag.data_ptr())
    eng.sync()
    a6 = eng.accum()
    for f in (7, 8):  # queued without a sync in between
        eng.frame_device(pos_d[f].data_ptr(), cell)
        eng.placements_device(1, tag.data_ptr())
    with pytest.raises(_lib.ErmodError) as ei:
        eng.sync()
    assert ei.value.code == _lib.E_ENG_SFT
    a = eng.accum()
    assert a["engnorm"] == a6["engnorm"] and np.array_equal(a["edens"], a6["edens"])
    eng.frame_device(pos_d[8].data_ptr(), cell)  # a new sequence after the sync
    eng.placements_device(1, tag.data_ptr())
    eng.sync()
    assert eng.accum()["engnorm"] == 2.0 * a6["engnorm"]  # one more placement of the same weight
    eng.close()


@pytest.mark.parametrize("K,order", [(40, 4), (45, 6), (48, 4), (64, 6), (72, 8), (96, 8), (100, 4), (125, 6), (128, 4),
                                     (144, 4)])
def test_compile_time_grid_sizes(gpu_lib, oracle, K, order):
    """Cubic grids with compile-time transforms (an odd one among them) against the
    oracle, with spline orders 4, 6 and 8 (other grids take the generic kernels)."""
    w = helpers.small_refs(K=K, corrcal=0, wgtslf=0)
    w.params["splodr"] = order
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(gpu_lib, oracle, w, topo, bins, "mixed")
    pos, cell = w.frame(0)
    pl = w.placements(0, 12)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    orc.frame(pos, cell)
    ro = orc.placements(tag, pl)
    gpu.frame(pos, cell)
    rg = gpu.placements(tag, pl, want_uvengy=True)
    _check_energies(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], "mixed")
    np.testing.assert_allclose(rg["uvengy"][:, 0], ro["uvengy"][:, 0], rtol=1e-6, atol=1e-4)
    gpu.close()


def test_set_bins_rejects_unsorted_edges(gpu_lib):
    """binsearch (engproc.F90:927-957) needs each species' edges in increasing order."""
    from ermod_gb300 import _lib
    from ermod_gb300.engproc import EnergyRepresentation
    w = helpers.small_refs(corrcal=0, wgtslf=0)
    topo, bins = helpers.build_inputs(w)
    gpu = EnergyRepresentation(w.params, topo, bins, precision="mixed")
    bad = dict(bins)
    bad["uvcrd"] = np.array(bins["uvcrd"], np.float64).copy()
    bad["uvcrd"][10], bad["uvcrd"][11] = bad["uvcrd"][11], bad["uvcrd"][10]
    with pytest.raises(_lib.ErmodError) as ei:
        gpu.set_bins(bad)
    assert ei.value.code == _lib.E_PARAM
    gpu.close()
