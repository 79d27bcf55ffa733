"""The benchmark's own workloads at full size (GPU).

* refs_large (33,000 waters in a 99.5 A box, a 12-site solute, PME 96^3, ecorr on,
  wgtslf and NPT weights): 8 placements of frame 0 against the oracle in both precisions,
  per-molecule energies, per-placement histograms and edens/ecorr bin by bin; and all
  50,000 insertions of frame 0 on the mixed path, checked by size-independent
  invariants: every placement bins all 33,000 molecules, so sum(edens) = 33,000 engnorm,
  each ecorr row sums to 33,000 times that bin's edens, ecorr is symmetric, and the
  int64 count mirror is symmetric and sums to exactly 50,000 x 33,000^2.
* refs_small at its own size (4,000 waters in a 49.3 A box, the 6-site solute, PME 48^3,
  ecorr on, weighted): 256 insertions of a frame against the oracle, per placement.
* soln_small (1,000 waters, PME 32^3, solution mode): several frames against the oracle.
"""
import numpy as np
import pytest

from tests import helpers
from tests.test_parity_gpu import _check_weighted

pytestmark = pytest.mark.gpu


def _setup(name, precision, **kw):
    from ermod_gb300 import setconf, synth
    from ermod_gb300.engproc import EnergyRepresentation
    w = synth.WORKLOADS[name]()
    topo = setconf.setparam_topology(w.species(), slttype=w.params["slttype"])
    bins = setconf.enginit_bins(topo["numslv"])
    return w, topo, bins, EnergyRepresentation(w.params, topo, bins, precision=precision, **kw)


def _against_oracle(oracle, name, precision, nplace, frames=(0,)):
    w, topo, bins, gpu = _setup(name, precision)
    orc = oracle.Oracle(w.params, topo, bins)
    uo_all = []
    for f in frames:
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        gpu.frame(pos, cell)
        if w.mode == "soln":
            tag, pl = [topo["nummol"]], None
        else:
            pl = w.placements(f, nplace)
            tag = np.full(len(pl), topo["nummol"], np.int32)
        ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True)
        uo, ug = ro["uvengy"], rg["uvengy"]
        band = helpers.mixed_band(w.solute) if precision == "mixed" else None
        err, err_soft = helpers.check_energies(ug[:, 1:], uo[:, 1:], precision, name, band=band)
        np.testing.assert_allclose(ug[:, 0], uo[:, 0], rtol=0, atol=helpers.self_tol(precision, w.solute))
        helpers.check_histograms(ug[:, 1:], uo[:, 1:], bins["uvcrd"], precision, f"{name} frame {f}", band=band)
        print(f"[parity] {name} {precision} frame {f}: max |du| {err:.3e} (|u| < 20: {err_soft:.3e}), "
              f"self energy max |du0| {np.abs(ug[:, 0] - uo[:, 0]).max():.3e}")
        uo_all.append(uo)
    ag, ao = gpu.accum(), orc.accum()
    if precision == "fp64":
        np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=1e-10)
        np.testing.assert_allclose(ag["edens"], ao["edens"], rtol=1e-10, atol=0)
        if ao["ecorr"] is not None:
            np.testing.assert_allclose(ag["ecorr"], ao["ecorr"], rtol=1e-10, atol=0)
    else:
        _check_weighted(ag, ao, np.concatenate(uo_all), bins["uvcrd"], w, corr=ao["ecorr"] is not None, label=name)
    gpu.close()
    orc.close()
    return w, topo


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_refs_large_against_oracle(gpu_lib, oracle, precision):
    w, topo = _against_oracle(oracle, "refs_large", precision, 8)
    assert topo["nummol"] - 1 == 33000 and w.params["ms1max"] == 96


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_refs_small_full_size_against_oracle(gpu_lib, oracle, precision):
    w, topo = _against_oracle(oracle, "refs_small", precision, 256)
    assert topo["nummol"] - 1 == 4000 and w.params["ms1max"] == 48 and w.params["corrcal"] == 1


def test_soln_small_frames_full_size(gpu_lib, oracle):
    _against_oracle(oracle, "soln_small", "mixed", 1, frames=range(8))


def test_refs_large_full_frame_invariants(gpu_lib):
    w, topo, bins, gpu = _setup("refs_large", "mixed", batch=256, count_mirror=True)
    pos, cell = w.frame(0)
    gpu.frame(pos, cell)
    n = w.ins_per_frame
    assert n == 50000
    pl = w.placements(0, n)
    gpu.placements(np.full(n, topo["nummol"], np.int32), pl)
    a = gpu.accum(with_count=True)
    nmol = gpu.slvmax
    assert a["engsmpl"] == n
    np.testing.assert_allclose(a["edens"].sum(), nmol * a["engnorm"], rtol=1e-12)
    ec = a["ecorr"]
    np.testing.assert_allclose(ec.sum(axis=1), nmol * a["edens"], rtol=1e-9, atol=1e-9 * np.abs(ec).max())
    # (w h_p) h_q and (w h_q) h_p round apart in the last bits, as FP64 products do
    np.testing.assert_allclose(ec, ec.T, rtol=1e-12, atol=1e-14 * np.abs(ec).max())
    cnt = a["ecorr_count"]
    assert int(cnt.sum()) == n * nmol * nmol
    np.testing.assert_array_equal(cnt, cnt.T)
    gpu.close()
