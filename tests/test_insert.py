"""Placements generated on the device (insertion.F90 modes, Philox4x32-10 stream).

CPU: the NumPy restatement's Philox against the published Philox4x32-10 known-answer
vectors.  GPU (marked gpu): the device generator against the restatement, placement by
placement (|dx| <= 1e-11 A), rigid-body distances preserved, mode geometry."""
import numpy as np
import pytest

from tests import insert_ref


def test_philox_known_answers():
    assert insert_ref.philox4x32_10((0, 0, 0, 0), (0, 0)) == (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)
    assert insert_ref.philox4x32_10((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2) == \
        (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)
    assert insert_ref.philox4x32_10((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0)) == \
        (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [dict(insposition=0), dict(insposition=2, lwreg=3.0, upreg=9.0),
                                  dict(insposition=4, lwreg=2.0, upreg=6.0), dict(insposition=5, upreg=2.0),
                                  dict(insposition=6, upreg=5.0), dict(insposition=1, insorient=1, insorigin=1)])
def test_device_placements_match_restatement(gpu_lib, mode):
    from ermod_gb300 import setconf, synth
    from ermod_gb300.engproc import EnergyRepresentation
    w = synth.refs_small()
    w.nwater, w.lattice_n, w.box = 300, 7, 22.0
    topo, bins = setconf.setparam_topology(w.species(), slttype=2), None
    bins = setconf.enginit_bins(topo["numslv"])
    eng = EnergyRepresentation(w.params, topo, bins, precision="mixed", batch=8)
    pos, cell = w.frame(0)
    eng.frame(pos, cell)
    bf = w.solute["xyz"] + np.array([1.0, -2.0, 0.5])
    mass = np.asarray(w.solute["mass"], float)
    n = 300
    sol, sws = eng.generate_placements(n, bf, mass, seed=12345, offset=77, weights=True, **mode)
    sol, sws = sol.cpu().numpy(), sws.cpu().numpy()
    for p in range(0, n, 7):
        x, wt = insert_ref.place(bf, mass, cell, p, seed=12345, offset=77, **mode)
        np.testing.assert_allclose(sol[p], x, atol=1e-11, rtol=0)
        np.testing.assert_allclose(sws[p], wt, rtol=1e-12)
    d0 = np.linalg.norm(bf[:, None] - bf[None], axis=-1)
    d = np.linalg.norm(sol[:, :, None] - sol[:, None, :], axis=-1)
    np.testing.assert_allclose(d, np.broadcast_to(d0, d.shape), atol=1e-10)
    com = (mass[None, :, None] * sol).sum(1) / mass.sum()
    if mode["insposition"] == 0:
        frac = com / w.box
        assert np.all((frac >= 0) & (frac < 1)) and abs(frac.mean() - 0.5) < 0.05
    if mode["insposition"] == 2:
        r = np.linalg.norm(com, axis=1)
        assert np.all((r >= 3.0 - 1e-9) & (r <= 9.0 + 1e-9))
    if mode["insposition"] == 4:
        assert np.all((np.abs(com[:, 2]) >= 2.0 - 1e-9) & (np.abs(com[:, 2]) <= 6.0 + 1e-9))
    # the generated placements run through the engine like host-given ones
    tag = np.full(n, topo["nummol"], np.int32)
    if mode["insposition"] in (0, 6):
        eng.placements(tag, sol)
    eng.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [dict(insposition=2, lwreg=2.0, upreg=6.0, insorigin=2),
                                  dict(insposition=4, lwreg=1.0, upreg=5.0, insorigin=2),
                                  dict(insposition=5, lwreg=0.0, upreg=2.5, insorigin=3),
                                  dict(insposition=6, lwreg=0.0, upreg=3.0, insorigin=3)])
def test_device_placements_aggregate_and_reference(gpu_lib, mode):
    """insorigin 2 (the solute's COM moved to the host aggregate's) and 3 (reffit: the solute
    fitted onto the reference solute carried into the frame, and the RMSD acceptance of
    check_solute_configuration, redrawing until it passes) against the restatement, whose
    fits use numpy's LAPACK eigensolver."""
    from ermod_gb300 import setconf, synth
    from ermod_gb300.engproc import EnergyRepresentation
    w = synth.refs_small()
    w.nwater, w.lattice_n, w.box = 300, 7, 22.0
    topo = setconf.setparam_topology(w.species(), slttype=2)
    bins = setconf.enginit_bins(topo["numslv"])
    eng = EnergyRepresentation(w.params, topo, bins, precision="mixed", batch=8)
    pos, cell = w.frame(0)
    eng.frame(pos, cell)
    mbi = np.asarray(topo["mol_begin_index"])
    mass_all = np.concatenate([np.tile(synth.WATER_MASS, w.nwater), w.solute["mass"]])
    host = np.zeros(topo["nummol"], np.int32)
    host[np.argsort(np.linalg.norm(pos[mbi[:-2] - 1] - w.box / 2, axis=1))[:12]] = 1
    hidx = np.concatenate([np.arange(mbi[i] - 1, mbi[i + 1] - 1) for i in np.nonzero(host)[0]])
    bf = w.solute["xyz"] + np.array([1.0, -2.0, 0.5])
    mass = np.asarray(w.solute["mass"], float)
    kw = {}
    if mode["insorigin"] == 2:
        eng.set_aggregate(host, mass_all)
        kw["agg"] = (mass_all[hidx, None] * pos[hidx]).sum(0) / mass_all[hidx].sum()
    else:
        th = 0.4
        R = np.array([[np.cos(th), 0.0, np.sin(th)], [0.0, 1.0, 0.0], [-np.sin(th), 0.0, np.cos(th)]])
        hc = pos[hidx] @ R.T + np.array([-2.0, 1.0, 4.0])
        hw = np.where(mass_all[hidx] > 0.95 * 4.0026, 1.0, 0.0)
        sc = w.solute["xyz"] - w.solute["xyz"].mean(0) + np.array([0.5, 0.0, -0.5])
        sw = np.where(mass > 0.95 * 4.0026, 1.0, 0.5)  # every site weighted: a unique fit
        eng.set_reference_structure(host, hc, hw, sc, sw)
        best = insert_ref.horn_fit(pos[hidx], hc, hw, sc)
        kw.update(start=insert_ref.horn_fit(best, bf, sw, bf), refbest=best, refw=sw)
    n = 120
    sol, sws = eng.generate_placements(n, bf, mass, seed=777, offset=5, weights=True, **mode)
    sol, sws = sol.cpu().numpy(), sws.cpu().numpy()
    for p in range(0, n, 5):
        x, wt = insert_ref.place(bf, mass, cell, p, seed=777, offset=5, **mode, **kw)
        np.testing.assert_allclose(sol[p], x, atol=1e-9, rtol=0)
        np.testing.assert_allclose(sws[p], wt, rtol=1e-10)
    com = (mass[None, :, None] * sol).sum(1) / mass.sum()
    if mode["insorigin"] == 2 and mode["insposition"] == 2:
        r = np.linalg.norm(com - kw["agg"], axis=1)
        assert np.all((r >= 2.0 - 1e-9) & (r <= 6.0 + 1e-9))
    if mode["insorigin"] == 3:  # every placement passed the acceptance
        rmsd = np.sqrt((sw * ((sol - kw["refbest"]) ** 2).sum(2)).sum(1) / sw.sum())
        assert np.all(rmsd <= mode["upreg"] + 1e-12)
    eng.close()


@pytest.mark.parametrize("nconf,nwt,pattern", [(5, 3, "11111"), (7, 0, "0110100"), (4, 9, "0001"),
                                               (6, 6, "101010")])
def test_library_closed_form_matches_getsolute_loop(nconf, nwt, pattern):
    """The device's closed form for the g-th accepted read (structure acc[g mod na] of file
    pass g / na, weight line r mod nweight) against getsolute's read loop itself."""
    accepted = [c == "1" for c in pattern]
    acc = [f for f in range(nconf) if accepted[f]]
    loop = insert_ref.library_reads(60, nconf, accepted, nwt)
    assert [insert_ref.library_pick(g, nconf, acc, nwt) for g in range(60)] == loop


def _library_engine():
    from ermod_gb300 import setconf, synth
    from ermod_gb300.engproc import EnergyRepresentation
    w = synth.refs_small()
    w.nwater, w.lattice_n, w.box = 300, 7, 22.0
    topo = setconf.setparam_topology(w.species(), slttype=2)
    bins = setconf.enginit_bins(topo["numslv"])
    eng = EnergyRepresentation(w.params, topo, bins, precision="mixed", batch=8)
    pos, cell = w.frame(0)
    eng.frame(pos, cell)
    rng = np.random.default_rng(31)
    base = w.solute["xyz"] + np.array([1.0, -2.0, 0.5])
    conf = base[None] + rng.normal(0.0, 0.35, (9,) + base.shape)  # a flexible solute's structures
    return w, topo, eng, pos, cell, conf


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [dict(insposition=0, nwt=3, insstructure=0),
                                  dict(insposition=6, upreg=5.0, nwt=7, insstructure=1),
                                  dict(insposition=5, lwreg=0.0, upreg=2.5, insorigin=3, nwt=0, insstructure=0)])
def test_device_placements_from_structure_library(gpu_lib, mode):
    """A flexible solute (getsolute): placement g takes the g-th accepted structure of the
    wrapped library and the weight read with it, then the rigid steps as before (insorigin 3
    fits each placement's own structure onto the reference solute in the frame)."""
    from ermod_gb300 import synth
    mode = dict(mode)
    nwt, insstructure = mode.pop("nwt"), mode.pop("insstructure")
    w, topo, eng, pos, cell, conf = _library_engine()
    mass = np.asarray(w.solute["mass"], float)
    # every site weighted: with two weighted sites the fit of a non-rigid copy is not unique
    # (any rotation about their axis fits as well)
    sw = np.where(mass > 0.95 * 4.0026, 1.0, 0.5)
    sc = w.solute["xyz"] - w.solute["xyz"].mean(0) + np.array([0.5, 0.0, -0.5])
    kw = {}
    if insstructure or mode.get("insorigin") == 3:
        mbi = np.asarray(topo["mol_begin_index"])
        mass_all = np.concatenate([np.tile(synth.WATER_MASS, w.nwater), w.solute["mass"]])
        host = np.zeros(topo["nummol"], np.int32)
        host[np.argsort(np.linalg.norm(pos[mbi[:-2] - 1] - w.box / 2, axis=1))[:12]] = 1
        hidx = np.concatenate([np.arange(mbi[i] - 1, mbi[i + 1] - 1) for i in np.nonzero(host)[0]])
        th = 0.4
        R = np.array([[np.cos(th), 0.0, np.sin(th)], [0.0, 1.0, 0.0], [-np.sin(th), 0.0, np.cos(th)]])
        hc = pos[hidx] @ R.T + np.array([-2.0, 1.0, 4.0])
        hw = np.where(mass_all[hidx] > 0.95 * 4.0026, 1.0, 0.0)
        eng.set_reference_structure(host, hc, hw, sc, sw)
        best = insert_ref.horn_fit(pos[hidx], hc, hw, sc)
    lw = up = 0.0
    if insstructure:  # a window that keeps some structures and rejects others, no RMSD near a bound
        r = np.sort([insert_ref.rmsd_bestfit(sc, x, sw) for x in conf])
        lw, up = 0.5 * (r[1] + r[2]), 0.5 * (r[6] + r[7])
        assert min(np.abs(r - lw).min(), np.abs(r - up).min()) > 1e-6
    wt = np.linspace(0.5, 2.0, nwt) if nwt else None
    eng.set_solute_library(conf, wt, insstructure=insstructure, lwstr=lw, upstr=up)
    acc = insert_ref.library_accepted(conf, insstructure, lw, up, sc, sw)
    assert 0 < len(acc) <= len(conf) and (len(acc) < len(conf)) == bool(insstructure)
    n, off = 90, 11
    sol, sws = eng.generate_placements(n, None, mass, seed=4242, offset=off, weights=True, **mode)
    sol, sws = sol.cpu().numpy(), sws.cpu().numpy()
    for p in range(0, n, 4):
        f, wl = insert_ref.library_pick(off + p, len(conf), acc, nwt)
        if mode.get("insorigin") == 3:
            kw = dict(start=insert_ref.horn_fit(best, conf[f], sw, conf[f]), refbest=best, refw=sw)
        x, wgt = insert_ref.place(conf[f], mass, cell, p, seed=4242, offset=off, w0=1.0 if wl is None else wt[wl],
                                  **mode, **kw)
        np.testing.assert_allclose(sol[p], x, atol=1e-9, rtol=0)
        np.testing.assert_allclose(sws[p], wgt, rtol=1e-10)
        d0 = np.linalg.norm(conf[f][:, None] - conf[f][None], axis=-1)  # the structure moves rigidly
        np.testing.assert_allclose(np.linalg.norm(sol[p][:, None] - sol[p][None], axis=-1), d0, atol=1e-10)
    eng.close()


@pytest.mark.gpu
def test_structure_library_refusals(gpu_lib):
    """ins_siz for structures of another size than the solute or the reference solute; a
    window that accepts nothing is refused (getsolute would read forever); the library's
    removal restores the rigid solute."""
    from ermod_gb300 import _lib
    w, topo, eng, pos, cell, conf = _library_engine()
    mass = np.asarray(w.solute["mass"], float)
    eng.set_solute_library(conf)
    with pytest.raises(_lib.ErmodError) as ei:
        eng.generate_placements(4, None, np.ones(len(mass) + 1), seed=1)
    assert ei.value.code == _lib.E_INS_SIZ
    with pytest.raises(_lib.ErmodError) as ei:  # insstructure 1 without a reference structure
        eng.set_solute_library(conf, insstructure=1, lwstr=0.0, upstr=1.0)
    assert ei.value.code == _lib.E_PARAM
    sw = np.ones(len(mass))
    eng.set_reference_structure(np.zeros(topo["nummol"], np.int32), np.zeros((0, 3)), np.zeros(0),
                                conf[0][:-1], sw[:-1])
    with pytest.raises(_lib.ErmodError) as ei:
        eng.set_solute_library(conf, insstructure=1, lwstr=0.0, upstr=1.0)
    assert ei.value.code == _lib.E_INS_SIZ
    eng.set_reference_structure(np.zeros(topo["nummol"], np.int32), np.zeros((0, 3)), np.zeros(0), conf[0], sw)
    with pytest.raises(_lib.ErmodError) as ei:
        eng.set_solute_library(conf, insstructure=1, lwstr=50.0, upstr=60.0)
    assert ei.value.code == _lib.E_PARAM
    eng.set_solute_library(conf, insstructure=1, lwstr=0.0, upstr=1e-9)  # only conf[0] itself
    sol, _ = eng.generate_placements(6, None, mass, insposition=1, insorient=1, insorigin=1, seed=1)
    np.testing.assert_allclose(sol.cpu().numpy(), np.broadcast_to(conf[0], (6,) + conf[0].shape), atol=0)
    eng.set_solute_library(None)
    bf = w.solute["xyz"]
    sol, _ = eng.generate_placements(3, bf, mass, insposition=1, insorient=1, insorigin=1, seed=1)
    np.testing.assert_allclose(sol.cpu().numpy(), np.broadcast_to(bf, (3,) + bf.shape), atol=0)
    eng.close()
