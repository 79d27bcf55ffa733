"""Parameter variants against the oracle (GPU, both precisions):

* the four LJ forms of realcal.F90 (ljswitch 0-3: CHARMM / GROMACS potential switch,
  CHARMM / GROMACS force switch, :667-770);
* reference-solvent mode with a flexible solute (slttype 3: realcal_self for every
  placement, engproc.F90:716-730) and caller-given solute weights;
* selfcal = 1 (the eself histogram of the solute self energy, engproc.F90:786-800) with a
  frame weight stat_weight_system != 1;
* spline orders 6 and 8 on the plain FP64 path;
* an energy coordinate of about 5,000 bins (first edge -200 kcal/mol).
"""
import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu


def _engines(oracle, params, topo, bins, precision, **kw):
    from ermod_gb300.engproc import EnergyRepresentation
    return EnergyRepresentation(params, topo, bins, precision=precision, **kw), oracle.Oracle(params, topo, bins)


def _check(ug, uo, precision, edges=None, label=""):
    helpers.check_energies(ug, uo, precision, label)
    if edges is not None:
        helpers.check_histograms(ug, uo, edges, precision, label)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("ljswitch", [0, 1, 2, 3])
def test_lj_forms(gpu_lib, oracle, ljswitch, precision):
    w = helpers.small_refs(corrcal=0, wgtslf=0)
    w.params["ljswitch"] = ljswitch
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(oracle, w.params, topo, bins, precision)
    pos, cell = w.frame(0)
    pl = w.placements(0, 24)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    orc.frame(pos, cell)
    gpu.frame(pos, cell)
    ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True)
    _check(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision, bins["uvcrd"], f"ljswitch {ljswitch}")
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_flexible_solute_with_weights(gpu_lib, oracle, precision):
    """slttype 3: each placement's own conformation (sites jittered by 0.05 A), so
    realcal_self differs per placement; stat_weight_solute per placement."""
    w = helpers.small_refs(corrcal=1, wgtslf=1)
    w.params["slttype"] = 3
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(oracle, w.params, topo, bins, precision, batch=16)
    rng = np.random.default_rng(7)
    for f in range(2):
        pos, cell = w.frame(f)
        pl = w.placements(f, 40) + rng.normal(0.0, 0.05, (40, len(w.solute["charge"]), 3))
        sws = rng.uniform(0.5, 2.0, 40)
        tag = np.full(len(pl), topo["nummol"], np.int32)
        orc.frame(pos, cell)
        gpu.frame(pos, cell)
        ro = orc.placements(tag, pl, stat_weight_solute=sws)
        rg = gpu.placements(tag, pl, stat_weight_solute=sws, want_uvengy=True)
        _check(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision, bins["uvcrd"], "flexible solute")
        # the self energies differ between placements and match the oracle's
        assert np.ptp(ro["uvengy"][:, 0]) > 1e-3
        np.testing.assert_allclose(rg["uvengy"][:, 0], ro["uvengy"][:, 0], rtol=0,
                                   atol=helpers.self_tol(precision, w.solute))
    ag, ao = gpu.accum(), orc.accum()
    # the weights' relative error from the self energies (u0 and voffset)
    rtol = helpers.weight_rtol(precision, w.solute, w.params["temp"])
    for key in ("engnorm", "avslf"):
        np.testing.assert_allclose(ag[key], ao[key], rtol=rtol)
    np.testing.assert_allclose(ag["edens"].sum(), ao["edens"].sum(), rtol=rtol)
    np.testing.assert_allclose(ag["ecorr"].sum(), ao["ecorr"].sum(), rtol=rtol)
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_selfcal_and_frame_weight(gpu_lib, oracle, precision):
    w = helpers.small_refs(corrcal=0, wgtslf=1)
    w.params["selfcal"] = 1
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(oracle, w.params, topo, bins, precision)
    pos, cell = w.frame(0)
    pl = w.placements(0, 32)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    orc.frame(pos, cell, stat_weight_system=0.37)
    gpu.frame(pos, cell, stat_weight_system=0.37)
    ro = orc.placements(tag, pl)
    gpu.placements(tag, pl)
    ag, ao = gpu.accum(), orc.accum()
    rtol = helpers.weight_rtol(precision, w.solute, w.params["temp"])
    np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=rtol)
    np.testing.assert_allclose(ag["avslf"], ao["avslf"], rtol=1e-12)
    np.testing.assert_allclose(ag["eself"].sum(), ao["eself"].sum(), rtol=rtol)
    assert np.count_nonzero(ao["eself"]) > 0
    # eself bin by bin: a self energy within the self-energy tolerance of an escrd edge
    # may take the neighbouring bin
    u0 = ro["uvengy"][:, 0]
    e = np.exp(-(u0 - u0[0]) / w.params["temp"])
    b_es, _ = helpers.weighted_bounds(u0[:, None], ao["engnorm"] * e / e.sum(), np.asarray(bins["escrd"]),
                                      helpers.self_tol(precision, w.solute), rtol)
    assert np.all(np.abs(ag["eself"] - ao["eself"]) <= b_es + 1e-12 * np.abs(ao["eself"]))
    gpu.close()


@pytest.mark.parametrize("order", [6, 8])
def test_fp64_spline_orders(gpu_lib, oracle, order):
    w = helpers.small_refs(corrcal=0, wgtslf=0)
    w.params["splodr"] = order
    topo, bins = helpers.build_inputs(w)
    gpu, orc = _engines(oracle, w.params, topo, bins, "fp64")
    pos, cell = w.frame(0)
    pl = w.placements(0, 6)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    orc.frame(pos, cell)
    gpu.frame(pos, cell)
    ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True)
    _check(rg["uvengy"], ro["uvengy"], "fp64")
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_large_energy_coordinate(gpu_lib, oracle, precision):
    """A first edge at -200 kcal/mol (about 5,000 bins): the finish kernel then counts
    straight into global memory instead of shared-memory block histograms.  Unit weights,
    so edens and the int64 ecorr counts are exact off the bin edges."""
    from ermod_gb300 import setconf
    w = helpers.small_refs(corrcal=1, wgtslf=0)
    w.params["estype"] = 1
    hist = dict(setconf.HIST_DEFAULT, ecdmin=-200.0)
    topo, bins = helpers.build_inputs(w, hist)
    assert len(bins["uvcrd"]) > 4000  # G x ermax x 4 B > 64 KB: global-memory counts
    gpu, orc = _engines(oracle, w.params, topo, bins, precision, count_mirror=True)
    pos, cell = w.frame(0)
    pl = w.placements(0, 48)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    orc.frame(pos, cell)
    gpu.frame(pos, cell)
    ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True)
    ug, uo = rg["uvengy"][:, 1:], ro["uvengy"][:, 1:]
    _check(ug, uo, precision)
    # the device's own bins of its own energies (unit weights: edens = summed counts)
    edges = np.asarray(bins["uvcrd"])
    model = sum(helpers.histogram(u, edges) for u in ug).astype(np.float64)
    ag, ao = gpu.accum(with_count=True), orc.accum()
    np.testing.assert_array_equal(ag["edens"], model)
    np.testing.assert_allclose(ag["edens"].sum(), ao["edens"].sum(), rtol=1e-12)
    # the int64 count mirror is the exact sum of count products
    h = np.stack([helpers.histogram(u, edges) for u in ug]).astype(np.int64)
    np.testing.assert_array_equal(ag["ecorr_count"], h.T @ h)
    gpu.close()
