"""Several systems of uneven size in one CUDA graph (marked gpu).

Three reference-mode systems (different boxes, grids and solutes) run step 0 through
ordinary calls and step 1 as one graph launch over all three; the accumulators must be
bit-identical to two ordinary steps per system (the graph holds the same kernels in the
same per-system order).  A second launch, with step 0's inputs written into the
captured buffers, adds its placements again.
"""
import numpy as np
import pytest

from ermod_gb300 import setconf, synth

pytestmark = pytest.mark.gpu


def _systems():
    out = []
    for i, (nw, nsite, ins) in enumerate(((300, 6, 40), (700, 9, 24), (1200, 14, 36))):
        rng = np.random.default_rng((77, i))
        box = (nw / 0.0334) ** (1.0 / 3.0)
        K = synth.fft_friendly(int(np.ceil(box)))
        sol = synth.random_solute(rng, nsite)
        lat = int(np.ceil(nw ** (1.0 / 3.0)))
        out.append(synth.Workload(f"g{i}", "refs", box, nw, sol, synth._params(2, K, corrcal=1, wgtslf=1),
                                  100 + i, 2, ins, lat))
    return out


def _build(w):
    from ermod_gb300.engproc import EnergyRepresentation
    topo = setconf.setparam_topology(w.species(), slttype=2)
    bins = setconf.enginit_bins(topo["numslv"])
    return EnergyRepresentation(w.params, topo, bins, precision="mixed", batch=8), topo


def test_graph_of_systems_matches_ordinary_calls(gpu_lib):
    from ermod_gb300.multisystem import SystemGraph
    ws = _systems()
    ref, topos = [], []
    for w in ws:  # ordinary calls: steps 0 and 1
        eng, topo = _build(w)
        tag = np.full(w.ins_per_frame, topo["nummol"], np.int32)
        for f in range(2):
            pos, cell = w.frame(f)
            eng.frame(pos, cell)
            eng.placements(tag, w.placements(f))
        ref.append(eng.accum())
        eng.close()
        topos.append(topo)
    engines = []
    for w, topo in zip(ws, topos):  # step 0 ordinary (it also sizes buffers and attributes)
        eng, _ = _build(w)
        pos, cell = w.frame(0)
        eng.frame(pos, cell)
        eng.placements(np.full(w.ins_per_frame, topo["nummol"], np.int32), w.placements(0))
        engines.append(eng)
    g = SystemGraph(engines, [w.frame(1) for w in ws], [w.placements(1) for w in ws],
                    [t["nummol"] for t in topos])
    g.launch()
    g.sync()
    for eng, r in zip(engines, ref):
        a = eng.accum()
        for k in ("edens", "ecorr", "eself", "minuv", "maxuv"):
            np.testing.assert_array_equal(a[k], r[k], err_msg=k)
        for k in ("engnorm", "engsmpl", "avslf", "voffset"):
            assert a[k] == r[k], k
    for i, w in enumerate(ws):
        g.set_frame(i, w.frame(0)[0])
        g.set_placements(i, w.placements(0))
    g.launch()
    g.sync()
    for eng, w in zip(engines, ws):
        assert eng.accum()["engsmpl"] == 3 * w.ins_per_frame
    g.close()
    for eng in engines:
        eng.close()


def test_tile_shapes_give_identical_results(gpu_lib):
    """The autotuner's tile shapes change the work split, not the arithmetic: finish groups 4
    and 8 and batches 8 and 16 give bit-identical energies and accumulators (ecorr: for
    equal batches), and autotune_tiles returns one of its candidates with a rate for each."""
    from ermod_gb300.engproc import EnergyRepresentation
    from ermod_gb300.multisystem import autotune_tiles
    w = _systems()[1]
    topo = setconf.setparam_topology(w.species(), slttype=2)
    bins = setconf.enginit_bins(topo["numslv"])
    pos, cell = w.frame(0)
    pl = w.placements(0, 24)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    out = []
    for B, G in ((8, 8), (8, 4), (16, 4), (16, 8)):
        eng = EnergyRepresentation(w.params, topo, bins, precision="mixed", batch=B, finish_group=G)
        eng.frame(pos, cell)
        r = eng.placements(tag, pl, want_uvengy=True)
        out.append((r["uvengy"], eng.accum()))
        eng.close()
    for u, a in out[1:]:
        np.testing.assert_array_equal(u, out[0][0])
        for key in ("edens", "engnorm", "minuv", "maxuv", "voffset"):
            np.testing.assert_array_equal(a[key], out[0][1][key], err_msg=key)
    # ecorr's float-float ring flushes follow the batch: equal for equal batches
    np.testing.assert_array_equal(out[1][1]["ecorr"], out[0][1]["ecorr"])
    np.testing.assert_array_equal(out[3][1]["ecorr"], out[2][1]["ecorr"])
    B, G, rates = autotune_tiles(w.params, topo, bins, (pos, cell), pl, topo["nummol"], batches=(8, 16), groups=(4, 8))
    assert (B, G) in rates and set(rates) == {(8, 4), (8, 8), (16, 4), (16, 8)}
    assert all(v > 0 for v in rates.values())


@pytest.mark.parametrize("adjoint", [False, True])
def test_graph_of_a_solution_mode_system(gpu_lib, adjoint):
    """A solution-mode system (ecorr off, the in-frame solute; the benchmark's form of a
    launch-bound step) captured alone: frame 1 as a graph launch after an ordinary frame 0
    gives the accumulators (and the adjoint sums) of two ordinary frames, bit for bit."""
    from ermod_gb300.engproc import EnergyRepresentation
    from ermod_gb300.multisystem import SystemGraph
    w = synth.soln_small(frames=3)
    topo = setconf.setparam_topology(w.species(), slttype=1)
    bins = setconf.enginit_bins(topo["numslv"], w.hist)
    tag = [topo["nummol"]]

    def make():
        eng = EnergyRepresentation(w.params, topo, bins, precision="mixed")
        if adjoint:
            eng.adjoint_enable()
        eng.frame(*w.frame(0))
        eng.placements(tag)
        return eng

    ref = make()
    ref.frame(*w.frame(1))
    ref.placements(tag)
    a_ref = ref.accum()
    g_ref = ref.adjoint_get() if adjoint else None
    ref.close()
    eng = make()
    g = SystemGraph([eng], [w.frame(1)], [None], tag)
    g.launch()
    g.sync()
    a = eng.accum()
    for k in ("edens", "eself", "slnuv", "minuv", "maxuv"):
        np.testing.assert_array_equal(a[k], a_ref[k], err_msg=k)
    for k in ("engnorm", "engsmpl", "avslf"):
        assert a[k] == a_ref[k], k
    if adjoint:
        gr, wt = eng.adjoint_get()
        np.testing.assert_array_equal(gr, g_ref[0])
        np.testing.assert_array_equal(wt, g_ref[1])
    g.close()
    eng.close()
