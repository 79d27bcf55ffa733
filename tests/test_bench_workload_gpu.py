"""The benchmark's own workload at full size (GPU): 33,000 waters in a 99.5 A box, a
12-site solute, PME 96^3, ecorr on, wgtslf and NPT weights.

* 8 placements of frame 0 against the oracle, both precisions;
* all 50,000 insertions of frame 0 on the mixed path, checked by size-independent
  invariants: every placement bins all 33,000 molecules, so sum(edens) = 33,000 engnorm,
  each ecorr row sums to 33,000 times that bin's edens, ecorr is symmetric, and the
  int64 count mirror is symmetric and sums to exactly 50,000 x 33,000^2.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(precision, **kw):
    from ermod_gb300 import setconf, synth
    from ermod_gb300.engproc import EnergyRepresentation
    w = synth.refs_large()
    topo = setconf.setparam_topology(w.species(), slttype=w.params["slttype"])
    bins = setconf.enginit_bins(topo["numslv"])
    return w, topo, bins, EnergyRepresentation(w.params, topo, bins, precision=precision, **kw)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_refs_large_against_oracle(gpu_lib, oracle, precision):
    w, topo, bins, gpu = _setup(precision)
    assert gpu.slvmax == 33000 and w.params["ms1max"] == 96
    orc = oracle.Oracle(w.params, topo, bins)
    pos, cell = w.frame(0)
    orc.frame(pos, cell)
    gpu.frame(pos, cell)
    pl = w.placements(0, 8)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True)
    atol, rtol = (1e-9, 1e-11) if precision == "fp64" else (1e-4, 2e-6)
    uo, ug = ro["uvengy"][:, 1:], rg["uvengy"][:, 1:]
    huge = np.abs(uo) >= 1e10
    assert np.all(ug[huge] >= 1e10)
    err = np.abs(ug - uo)[~huge]
    assert np.all(err <= atol + rtol * np.abs(uo[~huge])), f"max err {err.max():.3e}"
    ag, ao = gpu.accum(), orc.accum()
    wtol = 1e-10 if precision == "fp64" else 5e-4  # FP32-based self energies in the weights
    np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=wtol)
    np.testing.assert_allclose(ag["edens"].sum(), ao["edens"].sum(), rtol=wtol)
    np.testing.assert_allclose(ag["ecorr"].sum(), ao["ecorr"].sum(), rtol=wtol)
    gpu.close()


def test_refs_large_full_frame_invariants(gpu_lib):
    w, topo, bins, gpu = _setup("mixed", batch=256, count_mirror=True)
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
