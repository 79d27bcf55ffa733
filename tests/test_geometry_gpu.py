"""Geometry variants against the oracle (GPU, both precisions):

* an orthorhombic box (24 x 28 x 32 A) with a non-cubic PME grid (30 x 32 x 36): the
  generic transform kernels, per-axis fixed-point scales and B-spline moduli;
* non-cubic grids with K2 != K3 (one with odd K1) and many placements: each placement's
  self energy is the sum of its own K2 spectrum partials;
* solution mode with two solute molecules (sltlist of two entries; one placement per
  solute molecule, engproc.F90:677-684), each binned against the other as a solvent.
"""
import numpy as np
import pytest

from tests import helpers

pytestmark = pytest.mark.gpu


def _box_system(lengths, nwater, seed, solutes):
    """Waters on a jittered orthorhombic lattice plus the given solute molecules (each a
    dict of synth.random_solute form with a 'centre'); returns species, sitepos, cell."""
    from ermod_gb300 import insertion, synth
    rng = np.random.default_rng(seed)
    L = np.asarray(lengths, np.float64)
    n = np.ceil(L / 2.8).astype(int)  # ~2.8 A lattice spacing
    axes = [(np.arange(k) + 0.5) * (l / k) for k, l in zip(n, L)]
    pts = np.stack(np.meshgrid(*axes, indexing="ij"), -1).reshape(-1, 3)
    for s in solutes:
        pts = pts[np.linalg.norm(pts - s["centre"], axis=1) > 5.5]
    pts = pts[rng.choice(len(pts), nwater, replace=False)]
    body = synth.water_body() - insertion.center_of_mass(synth.water_body(), synth.WATER_MASS)
    q = insertion.random_quaternions(rng, nwater)
    wat = insertion.quat_rotate(q, np.broadcast_to(body, (nwater, 3, 3))) + (pts + rng.uniform(-0.3, 0.3, pts.shape))[:, None]
    parts = [wat.reshape(-1, 3)]
    species = [dict(count=nwater, sluvid=0, charge=synth.WATER_CHARGE, eps=synth.WATER_EPS, len=synth.WATER_SIG)]
    for s in solutes:
        parts.append(s["xyz"] - insertion.center_of_mass(s["xyz"], s["mass"]) + s["centre"])
    species.append(dict(count=len(solutes), sluvid=1, charge=solutes[0]["charge"], eps=solutes[0]["eps"],
                        len=solutes[0]["sig"]))
    return species, np.ascontiguousarray(np.concatenate(parts)), np.diag(L)


def _run(oracle, params, species, pos, cell, nsolute, precision):
    """One placement for each of the last nsolute molecules (the solutes), in order."""
    from ermod_gb300 import setconf
    from ermod_gb300.engproc import EnergyRepresentation
    topo = setconf.setparam_topology(species, slttype=params["slttype"])
    bins = setconf.enginit_bins(topo["numslv"])
    gpu = EnergyRepresentation(params, topo, bins, precision=precision)
    orc = oracle.Oracle(params, topo, bins)
    orc.frame(pos, cell)
    gpu.frame(pos, cell)
    tag = np.arange(topo["nummol"] - nsolute + 1, topo["nummol"] + 1, dtype=np.int32)
    ro = orc.placements(tag)
    rg = gpu.placements(tag, want_uvengy=True)
    helpers.check_energies(rg["uvengy"], ro["uvengy"], precision, "geometry")
    rep = helpers.check_histograms(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], bins["uvcrd"], precision, "geometry")
    ag, ao = gpu.accum(), orc.accum()
    np.testing.assert_allclose(ag["edens"].sum(), ao["edens"].sum(), rtol=1e-12)
    if rep["other_bin"] == 0:
        np.testing.assert_array_equal(ag["edens"], ao["edens"])
    gpu.close()
    return ro


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_orthorhombic_box_noncubic_grid(gpu_lib, oracle, precision):
    from ermod_gb300 import synth
    sol = synth.methanol_like()
    species, pos, cell = _box_system((24.0, 28.0, 32.0), 600, 41, [dict(sol, centre=np.array([12.0, 14.0, 16.0]))])
    params = synth._params(1, 32, corrcal=0, wgtslf=0)
    params.update(ms1max=30, ms2max=32, ms3max=36)
    _run(oracle, params, species, pos, cell, 1, precision)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_solution_two_solute_molecules(gpu_lib, oracle, precision):
    from ermod_gb300 import synth
    sol = synth.methanol_like()
    centres = [np.array([8.0, 13.0, 13.0]), np.array([18.0, 13.0, 13.0])]
    species, pos, cell = _box_system((26.0, 26.0, 26.0), 520, 43, [dict(sol, centre=c) for c in centres])
    params = synth._params(1, 32, corrcal=0, wgtslf=0)
    ro = _run(oracle, params, species, pos, cell, 2, precision)
    # each solute sees the other one as a solvent molecule (its slot is not the self slot)
    assert np.count_nonzero(ro["uvengy"][0, 1:]) == 520 + 1


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("grid", [(30, 32, 36), (45, 48, 50)])  # the second: odd K1, generic kernels
def test_noncubic_grid_self_energies(gpu_lib, oracle, precision, grid):
    from ermod_gb300.engproc import EnergyRepresentation
    w = helpers.small_refs(corrcal=0, wgtslf=0)
    w.params.update(ms1max=grid[0], ms2max=grid[1], ms3max=grid[2])
    topo, bins = helpers.build_inputs(w)
    gpu = EnergyRepresentation(w.params, topo, bins, precision=precision, batch=16)
    orc = oracle.Oracle(w.params, topo, bins)
    pos, cell = w.frame(0)
    orc.frame(pos, cell)
    gpu.frame(pos, cell)
    pl = w.placements(0, 20)
    tag = np.full(len(pl), topo["nummol"], np.int32)
    ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True)
    np.testing.assert_allclose(rg["uvengy"][:, 0], ro["uvengy"][:, 0], rtol=0, atol=helpers.self_tol(precision, w.solute))
    helpers.check_energies(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], precision, f"grid {grid}")
    helpers.check_histograms(rg["uvengy"][:, 1:], ro["uvengy"][:, 1:], bins["uvcrd"], precision, f"grid {grid}")
    gpu.close()
