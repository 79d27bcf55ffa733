"""GPU path vs the FP64 oracle, through the C ABI (marked gpu).

Tolerances: ``tests/helpers.py`` states them (per-molecule energies, the bin-edge band of
the mixed path, solute self energies) and derives the bin-by-bin bounds of the weighted
accumulators from them.  Histograms are exact for every molecule outside the band; the
molecules within 1e-6 and within the band of an edge and those binned elsewhere are
counted and printed.
"""
import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu


def _engines(gpu_lib, oracle, w, topo, bins, precision, **kw):
    from ermod_gb300.engproc import EnergyRepresentation
    gpu = EnergyRepresentation(w.params, topo, bins, precision=precision, **kw)
    orc = oracle.Oracle(w.params, topo, bins)
    return gpu, orc


def _check_energies(u_gpu, u_orc, precision, label=""):
    return helpers.check_energies(u_gpu, u_orc, precision, label)[1]


def _placement_weights(u0, engnorm, temp, wgtslf):
    """Each placement's engnmfc of one cell (the volume and charge factors are common to
    all placements, so the weights are exp(-(u0 - voffset)/kT) scaled to sum to engnorm)."""
    e = np.exp(-(u0 - u0[0]) / temp) if wgtslf else np.ones_like(u0)
    return engnorm * e / e.sum()


def _check_weighted(ag, ao, u_orc, edges, w, corr=True, label=""):
    """edens and ecorr bin by bin: the weights' relative error from the self energies,
    plus the weight of every near-edge molecule that may sit in a neighbouring bin."""
    precision = "mixed"
    rtol_w = helpers.weight_rtol(precision, w.solute, w.params["temp"])
    wts = _placement_weights(u_orc[:, 0], ao["engnorm"], w.params["temp"], w.params["wgtslf"])
    b_ed, b_ec = helpers.weighted_bounds(u_orc[:, 1:], wts, edges, helpers.mixed_band(w.solute), rtol_w, corr=corr)
    d_ed = np.abs(ag["edens"] - ao["edens"])
    assert np.all(d_ed <= b_ed + 1e-12 * np.abs(ao["edens"])), f"{label}: edens bin {int(np.argmax(d_ed - b_ed))}"
    if corr:
        d_ec = np.abs(ag["ecorr"] - ao["ecorr"])
        assert np.all(d_ec <= b_ec + 1e-12 * np.abs(ao["ecorr"])), f"{label}: ecorr entry {np.unravel_index(int(np.argmax(d_ec - b_ec)), d_ec.shape)}"
    np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=rtol_w)
    np.testing.assert_allclose(ag["voffset"], ao["voffset"], atol=helpers.self_tol(precision, w.solute))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_soln_small_frames(gpu_lib, oracle, precision):
    from ermod_gb300 import synth
    w = synth.soln_small()
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(gpu_lib, oracle, w, topo, bins, precision)
    tag = [topo["nummol"]]
    ug_all, uo_all = [], []
    for f in range(3):
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        ro = orc.placements(tag)
        gpu.frame(pos, cell)
        rg = gpu.placements(tag, want_uvengy=True, want_flceng=True)
        _check_energies(rg["uvengy"], ro["uvengy"], precision, "soln_small")
        np.testing.assert_allclose(rg["flceng"], ro["flceng"], atol=helpers.ENERGY_TOL[precision][0] * topo["nummol"],
                                   rtol=1e-9)
        ug_all.append(rg["uvengy"][:, 1:])
        uo_all.append(ro["uvengy"][:, 1:])
    edges = bins["uvcrd"]
    rep = helpers.check_histograms(np.concatenate(ug_all), np.concatenate(uo_all), edges, precision, "soln_small")
    ag, ao = gpu.accum(), orc.accum()
    if precision == "fp64" or rep["other_bin"] == 0:
        np.testing.assert_array_equal(ag["edens"], ao["edens"])
    for k in ("engnorm", "engsmpl", "avslf"):
        np.testing.assert_allclose(ag[k], ao[k], rtol=1e-12)
    np.testing.assert_allclose(ag["minuv"], ao["minuv"], atol=helpers.ENERGY_TOL[precision][0])
    np.testing.assert_allclose(ag["maxuv"], ao["maxuv"], atol=helpers.ENERGY_TOL[precision][0])
    # slnuv = sum of flceng * engnmfc (engnmfc = V here): the per-molecule tolerance summed
    np.testing.assert_allclose(ag["slnuv"], ao["slnuv"], rtol=0,
                               atol=topo["nummol"] * helpers.ENERGY_TOL[precision][0] * ag["engnorm"])
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
    _check_energies(rg["uvengy"], ro["uvengy"], precision, "refs unit weights")
    edges = bins["uvcrd"]
    ug, uo = rg["uvengy"][:, 1:], ro["uvengy"][:, 1:]
    rep = helpers.check_histograms(ug, uo, edges, precision, "refs unit weights")
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
    if precision == "fp64" or rep["other_bin"] == 0:
        np.testing.assert_array_equal(ag["edens"], ao["edens"])
        np.testing.assert_array_equal(ag["ecorr"], ao["ecorr"])
    else:  # unit weights: the bounds are the near-edge molecules' counts
        _check_weighted(ag, ao, ro["uvengy"], edges, w, label="refs unit weights")
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_refs_weighted_accumulators(gpu_lib, oracle, precision):
    """REFS defaults: wgtslf = 1, NPT; weights exp(-(u0 - voffset)/kT) V.  edens and ecorr
    are compared bin by bin (mixed: within the bounds the energy band and the self-energy
    tolerance give)."""
    w = helpers.small_refs()
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(gpu_lib, oracle, w, topo, bins, precision, batch=16)
    uo_all = []
    for f in range(2):
        pos, cell = w.frame(f)
        pl = w.placements(f, 40)
        tag = np.full(len(pl), topo["nummol"], np.int32)
        orc.frame(pos, cell)
        ro = orc.placements(tag, pl)
        gpu.frame(pos, cell)
        rg = gpu.placements(tag, pl, want_uvengy=True)
        _check_energies(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision, "refs weighted")
        helpers.check_histograms(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], bins["uvcrd"], precision, "refs weighted")
        # the solute self energy decides the weights
        np.testing.assert_allclose(rg["uvengy"][:, 0], ro["uvengy"][:, 0], rtol=0,
                                   atol=helpers.self_tol(precision, w.solute))
        uo_all.append(ro["uvengy"])
    ag, ao = gpu.accum(), orc.accum()
    np.testing.assert_allclose(ag["avslf"], ao["avslf"], rtol=1e-12)
    assert ag["engsmpl"] == ao["engsmpl"] == 80
    if precision == "fp64":
        np.testing.assert_allclose(ag["voffset"], ao["voffset"], atol=1e-9)
        np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=1e-10)
        np.testing.assert_allclose(ag["edens"], ao["edens"], rtol=1e-10, atol=0)
        np.testing.assert_allclose(ag["ecorr"], ao["ecorr"], rtol=1e-10, atol=0)
    else:
        _check_weighted(ag, ao, np.concatenate(uo_all), bins["uvcrd"], w, label="refs weighted")
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
    _check_energies(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], "mixed", f"K={K} order {order}")
    helpers.check_histograms(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], bins["uvcrd"], "mixed", f"K={K} order {order}")
    np.testing.assert_allclose(rg["uvengy"][:, 0], ro["uvengy"][:, 0], rtol=0, atol=helpers.self_tol("mixed", w.solute))
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
