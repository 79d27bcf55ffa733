"""Edge cases of the placement call (GPU, both precisions, against the oracle):

* an empty call (nplace 0) returns OK and leaves the accumulators untouched;
* ragged batches: 53 placements in batches of 16 (three full, one of 5) give the
  oracle's accumulators, and the same accumulators as one batch of 64;
* the largest solute, 256 sites (kMaxSoluteSites): the spectrum generation then runs
  over several site chunks; a 257-site solute is refused with ERMOD_E_UNSUPPORTED;
* the largest system of the 16-system set (58,329 waters, PME 125^3).
"""
import numpy as np
import pytest

from tests import helpers
from tests.test_parity_gpu import _check_weighted

pytestmark = pytest.mark.gpu


def _engine(w, precision, **kw):
    from ermod_gb300.engproc import EnergyRepresentation
    topo, bins = helpers.build_inputs(w)
    return EnergyRepresentation(w.params, topo, bins, precision=precision, **kw), topo, bins


def _check_uv(ug, uo, precision, edges=None, label="", solute=None):
    band = helpers.mixed_band(solute) if precision == "mixed" else None
    helpers.check_energies(ug, uo, precision, label, band=band)
    if edges is not None:
        helpers.check_histograms(ug, uo, edges, precision, label, band=band)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_empty_call(gpu_lib, oracle, precision):
    w = helpers.small_refs(corrcal=1, wgtslf=1)
    gpu, topo, bins = _engine(w, precision)
    pos, cell = w.frame(0)
    gpu.frame(pos, cell)
    ns = len(w.solute["charge"])
    r = gpu.placements(np.zeros(0, np.int32), np.zeros((0, ns, 3)), want_uvengy=True)
    assert r["uvengy"].shape == (0, gpu.slvmax + 1)
    a = gpu.accum()
    assert a["engnorm"] == 0.0 and a["engsmpl"] == 0.0
    assert not np.any(a["edens"]) and not np.any(a["ecorr"])
    # the context is still usable and gives the oracle's energies
    orc = oracle.Oracle(w.params, topo, bins)
    orc.frame(pos, cell)
    pl = w.placements(0, 8)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True)
    _check_uv(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision, bins["uvcrd"], "after an empty call")
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ragged_batches(gpu_lib, oracle, precision):
    w = helpers.small_refs(corrcal=1, wgtslf=1)
    g16, topo, bins = _engine(w, precision, batch=16)
    g64, _, _ = _engine(w, precision, batch=64)
    orc = oracle.Oracle(w.params, topo, bins)
    uo_all = []
    for f in range(2):
        pos, cell = w.frame(f)
        pl = w.placements(f, 53)
        tag = np.full(len(pl), topo["nummol"], np.int32)
        for e in (g16, g64, orc):
            e.frame(pos, cell)
        ro = orc.placements(tag, pl)
        r16 = g16.placements(tag, pl, want_uvengy=True)
        r64 = g64.placements(tag, pl, want_uvengy=True)
        _check_uv(r16["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision, bins["uvcrd"], "ragged batches")
        uo_all.append(ro["uvengy"])
        # the batch size does not change a placement's energies: bit for bit on the mixed
        # path (per-placement arithmetic); the FP64 path's cuFFT plans differ per batch size
        if precision == "mixed":
            np.testing.assert_array_equal(r16["uvengy"], r64["uvengy"])
        else:
            np.testing.assert_allclose(r16["uvengy"], r64["uvengy"], rtol=1e-12, atol=1e-10)
    a16, a64, ao = g16.accum(), g64.accum(), orc.accum()
    # wgtslf = 1: the weights follow the solute self energy
    if precision == "fp64":
        np.testing.assert_allclose(a16["engnorm"], ao["engnorm"], rtol=1e-10)
        np.testing.assert_allclose(a16["edens"], ao["edens"], rtol=1e-10, atol=0)
        np.testing.assert_allclose(a16["ecorr"], ao["ecorr"], rtol=1e-10, atol=0)
    else:
        _check_weighted(a16, ao, np.concatenate(uo_all), bins["uvcrd"], w, label="ragged batches")
    # one batch of 64 against batches of 16: the same sums in placement order (ecorr's
    # float-float flush groups differ on the mixed path)
    for key in ("edens", "engnorm", "avslf", "minuv", "maxuv"):
        np.testing.assert_allclose(a16[key], a64[key], rtol=1e-12, atol=1e-13 * np.abs(a64[key]).max())
    np.testing.assert_allclose(a16["ecorr"], a64["ecorr"], rtol=1e-12 if precision == "fp64" else 1e-9,
                               atol=1e-12 * np.abs(a64["ecorr"]).max())
    g16.close()
    g64.close()


def _big_solute_workload(nsite):
    """A compact solute of nsite sites; its charges are scaled to a quarter so that no
    water binds below the default first edge (-20 kcal/mol), where the reference stops."""
    from ermod_gb300 import synth
    sol = synth.random_solute(np.random.default_rng((5, nsite)), nsite)
    sol = dict(sol, charge=0.25 * np.asarray(sol["charge"]))
    return helpers.small_refs(nwater=1500, box=40.0, K=40, corrcal=0, wgtslf=0, solute=sol, lattice=12)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_largest_solute(gpu_lib, oracle, precision):
    w = _big_solute_workload(256)
    gpu, topo, bins = _engine(w, precision)
    orc = oracle.Oracle(w.params, topo, bins)
    pos, cell = w.frame(0)
    orc.frame(pos, cell)
    gpu.frame(pos, cell)
    pl = w.placements(0, 6)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True)
    _check_uv(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision, bins["uvcrd"], "256-site solute", w.solute)
    # the self energy (all 256 sites' spectrum, summed over the site chunks): about
    # -1 kcal/mol, net of reciprocal and real-space parts that largely cancel
    np.testing.assert_allclose(rg["uvengy"][:, 0], ro["uvengy"][:, 0], rtol=0,
                               atol=helpers.self_tol(precision, w.solute))
    gpu.close()


def test_solute_above_the_limit_is_refused(gpu_lib):
    from ermod_gb300 import _lib
    w = _big_solute_workload(257)
    gpu, topo, _ = _engine(w, "mixed")
    pos, cell = w.frame(0)
    gpu.frame(pos, cell)
    pl = w.placements(0, 2)
    with pytest.raises(_lib.ErmodError) as ex:
        gpu.placements(np.full(len(pl), topo["nummol"], np.int32), pl)
    assert ex.value.code == _lib.E_UNSUPPORTED
    gpu.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_largest_uneven_system(gpu_lib, oracle, precision):
    """The largest system of the 16-system set: 58,329 waters in a 120 A box, a 15-site
    solute and an energy coordinate from -200 kcal/mol (4,996 bins: global-memory counts in
    the finish kernel), with the grid set to 125^3 (three-pass transforms; the set itself
    rounds the box to 128^3)."""
    from ermod_gb300 import setconf, synth
    from ermod_gb300.engproc import EnergyRepresentation
    w = max(synth.uneven(), key=lambda x: x.nwater)
    assert w.nwater > 58000 and w.params["ms1max"] == 128
    w.params.update(ms1max=125, ms2max=125, ms3max=125)
    topo = setconf.setparam_topology(w.species(), slttype=w.params["slttype"])
    bins = setconf.enginit_bins(topo["numslv"], w.hist)
    gpu = EnergyRepresentation(w.params, topo, bins, precision=precision)
    orc = oracle.Oracle(w.params, topo, bins)
    pos, cell = w.frame(0)
    orc.frame(pos, cell)
    gpu.frame(pos, cell)
    pl = w.placements(0, 4)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True)
    _check_uv(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision, bins["uvcrd"], "58,329 waters", w.solute)
    np.testing.assert_allclose(rg["uvengy"][:, 0], ro["uvengy"][:, 0], rtol=0,
                               atol=helpers.self_tol(precision, w.solute))
    ag, ao = gpu.accum(), orc.accum()
    if precision == "fp64":
        np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=1e-10)
        np.testing.assert_allclose(ag["edens"], ao["edens"], rtol=1e-10, atol=0)
        np.testing.assert_allclose(ag["ecorr"], ao["ecorr"], rtol=1e-10, atol=0)
    else:
        _check_weighted(ag, ao, ro["uvengy"], bins["uvcrd"], w, label="58,329 waters")
    gpu.close()
