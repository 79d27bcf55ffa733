"""Solution-mode configuration check (check_mol_configuration, engproc.F90:1046-1100): a
placement whose solute lies outside [lwreg, upreg] of the host aggregate is skipped by the
placement loop (skipcond, engproc.F90:389-390) and accumulates nothing.

The system: waters on a lattice, ten methanol-like solute molecules (sluvid 1) spread
through the box, and a host aggregate of the twenty waters nearest the centre.  The
bounds are put between the solutes' distances (none within 1e-6 of a bound), so that a
few solutes are kept and a few rejected on each side.

CPU: the oracle with the check over all solutes equals the oracle without it over the
kept solutes alone, bit for bit; rejected rows are zero; slab checks of a non-periodic
system report eng_slb.  GPU (marked): both precisions against the oracle.
"""
import numpy as np
import pytest

from tests import helpers

NSLT = 10


def _system(seed=41, nwater=400, box=26.0, K=32, wgtslf=0, jitter=0.0):
    from ermod_gb300 import insertion, setconf, synth
    meoh = synth.methanol_like()
    rng = np.random.default_rng((seed, 5))
    n = 9
    g = (np.arange(n) + 0.5) * (box / n)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    # solutes on lattice points 5.5 A apart or more, waters only on points as clear of every
    # solute (overlaps would stop the run with soft-core errors)
    def mind(x, y):  # minimum-image distances
        d = x - y
        return np.linalg.norm(d - box * np.round(d / box), axis=-1)

    lat_s = []
    for i in rng.permutation(len(pts)):
        if all(mind(pts[i], q) > 5.5 for q in lat_s):
            lat_s.append(pts[i])
        if len(lat_s) == NSLT:
            break
    lat_s = np.array(lat_s)
    gap = mind(pts[:, None, :], lat_s[None, :, :]).min(1)
    free = np.nonzero(gap > 5.5)[0]
    lat_w = pts[np.sort(rng.choice(free, nwater, replace=False))]
    species = [dict(count=nwater, sluvid=0, charge=synth.WATER_CHARGE, eps=synth.WATER_EPS, len=synth.WATER_SIG),
               dict(count=NSLT, sluvid=1, charge=meoh["charge"], eps=meoh["eps"], len=meoh["sig"])]
    params = synth._params(1, K, corrcal=1, wgtslf=wgtslf, estype=1)
    topo = setconf.setparam_topology(species, slttype=1)
    bins = setconf.enginit_bins(topo["numslv"])
    cell = np.diag([box] * 3)
    mass = np.concatenate([np.tile(synth.WATER_MASS, nwater), np.tile(meoh["mass"], NSLT)])
    host = np.zeros(topo["nummol"], np.int32)
    host[np.argsort(np.linalg.norm(lat_w - box / 2, axis=1))[:20]] = 1
    solutes = np.arange(nwater + 1, nwater + NSLT + 1, dtype=np.int32)  # 1-based molecule numbers

    def place(body, m, centres, r):
        body = body - insertion.center_of_mass(body, m)
        q = insertion.random_quaternions(r, len(centres))
        return (insertion.quat_rotate(q, np.broadcast_to(body, (len(centres),) + body.shape))
                + centres[:, None, :]).reshape(-1, 3)

    def frame(i):
        r = np.random.default_rng((seed, 100 + i))
        w = place(synth.water_body(), synth.WATER_MASS, lat_w + r.uniform(-0.3, 0.3, lat_w.shape), r)
        s = place(meoh["xyz"], meoh["mass"], lat_s + r.uniform(-0.3, 0.3, lat_s.shape), r)
        if jitter:  # each solute's own distortion (the structure test sees different RMSDs)
            s = s + r.normal(0.0, jitter, s.shape)
        return np.ascontiguousarray(np.concatenate([w, s])), cell

    return params, topo, bins, frame, mass, host, solutes


def _reference(pos, topo, host, mass):
    """A reference structure: the host waters of frame 0 turned and moved by a fixed rigid
    motion (so that the fit has work to do), and the methanol-like solute's own geometry
    with read_refPDF_weight's default weights (1 for heavy atoms, 0 for hydrogens)."""
    from ermod_gb300 import synth
    mbi = np.asarray(topo["mol_begin_index"])
    idx = np.concatenate([np.arange(mbi[i] - 1, mbi[i + 1] - 1) for i in np.nonzero(host)[0]])
    th = 0.7
    R = np.array([[np.cos(th), -np.sin(th), 0.0], [np.sin(th), np.cos(th), 0.0], [0.0, 0.0, 1.0]])
    hc = pos[idx] @ R.T + np.array([5.0, -3.0, 2.0])
    hw = np.where(mass[idx] > 0.95 * 4.0026, 1.0, 0.0)
    meoh = synth.methanol_like()
    sc = meoh["xyz"] - meoh["xyz"].mean(0)
    sw = np.where(meoh["mass"] > 0.95 * 4.0026, 1.0, 0.0)
    return host.copy(), hc, hw, sc, sw


def _distances(pos, mass, topo, host, solutes, insposition, cell, ref=None, structure=False):
    """The check's distance of each solute (engproc.F90:1072-1141), in numpy (the fits with
    numpy's LAPACK eigensolver)."""
    from tests import insert_ref
    mbi = np.asarray(topo["mol_begin_index"])
    if insposition == 5 or structure:
        rm, hc, hw, sc, sw = ref
        hidx = np.concatenate([np.arange(mbi[i] - 1, mbi[i + 1] - 1) for i in np.nonzero(rm)[0]])
        best = insert_ref.horn_fit(pos[hidx], hc, hw, sc)
        out = []
        for t in solutes:
            x = pos[mbi[t - 1] - 1:mbi[t] - 1]
            if structure:
                fitted = insert_ref.horn_fit(sc, x, sw, x)
                out.append(np.sqrt((sw * ((fitted - sc) ** 2).sum(1)).sum() / sw.sum()))
            else:
                out.append(np.sqrt((sw * ((x - best) ** 2).sum(1)).sum() / sw.sum()))
        return np.array(out)

    def com(mols):
        idx = np.concatenate([np.arange(mbi[i] - 1, mbi[i + 1] - 1) for i in mols])
        return (pos[idx] * mass[idx, None]).sum(0) / mass[idx].sum()

    agg = com(np.nonzero(host)[0])
    dx = np.array([com([t - 1]) - agg for t in solutes])
    if insposition == 2:
        return np.linalg.norm(dx, axis=1)
    inv3 = np.linalg.inv(cell)[2]  # row 3 of the inverse cell (columns = cell vectors)
    d = (dx @ inv3) * np.linalg.norm(cell[:, 2])
    return np.abs(d) if insposition == 4 else d


def _bounds(d):
    """lwreg/upreg between the 2nd/3rd and 7th/8th smallest distances of the first frame."""
    s = np.sort(d)
    return 0.5 * (s[1] + s[2]), 0.5 * (s[6] + s[7])


def _configure(eng, check):
    """check = (aggregate (host_mol, sitemass) or None, reference structure or None,
    set_configuration_check arguments)."""
    agg, ref, args = check
    if agg is not None:
        eng.set_aggregate(*agg)
    if ref is not None:
        eng.set_reference_structure(*ref)
    eng.set_configuration_check(*args)


def _run_oracle(oracle, params, topo, bins, frames, tags, check=None):
    orc = oracle.Oracle(params, topo, bins)
    if check is not None:
        _configure(orc, check)
    out = []
    for (pos, cell), tg in zip(frames, tags):
        orc.frame(pos, cell)
        out.append(orc.placements(tg))
    a = orc.accum()
    orc.close()
    return out, a


def _setup(insposition, nframes=2, wgtslf=0, structure=False):
    """insposition 2-5 (the position test), or structure=True (insposition 0 with the
    structure test)."""
    params, topo, bins, frame, mass, host, solutes = _system(wgtslf=wgtslf, jitter=0.15 if structure else 0.0)
    frames = [frame(i) for i in range(nframes)]
    ref = _reference(frames[0][0], topo, host, mass)
    d0 = _distances(frames[0][0], mass, topo, host, solutes, insposition, frames[0][1], ref, structure)
    lw, up = _bounds(d0)
    keep = []
    for pos, cell in frames:
        d = _distances(pos, mass, topo, host, solutes, insposition, cell, ref, structure)
        assert np.min(np.abs(d - lw)) > 1e-6 and np.min(np.abs(d - up)) > 1e-6
        keep.append((lw <= d) & (d <= up))
    # the first placement of each frame a rejected one: voffset then comes from a later one
    order = [np.concatenate([np.nonzero(~k)[0], np.nonzero(k)[0]]) for k in keep]
    tags = [solutes[o] for o in order]
    keep = [k[o] for k, o in zip(keep, order)]
    for k in keep:
        assert 2 <= k.sum() <= NSLT - 2
    args = (0, 0.0, 0.0, 1, lw, up) if structure else (insposition, lw, up)
    agg = (host, mass) if 2 <= insposition <= 4 else None
    return params, topo, bins, frames, (agg, ref if (insposition == 5 or structure) else None, args), tags, keep


CASES = [dict(insposition=2), dict(insposition=3), dict(insposition=4), dict(insposition=5),
         dict(insposition=0, structure=True)]
CASE_IDS = ["sphere", "slab", "symmetric-slab", "rmsd", "structure"]


@pytest.mark.parametrize("case", CASES, ids=CASE_IDS)
def test_oracle_skip_equals_kept_only(oracle, case):
    params, topo, bins, frames, check, tags, keep = _setup(wgtslf=1, **case)
    r_chk, a_chk = _run_oracle(oracle, params, topo, bins, frames, tags, check)
    r_ref, a_ref = _run_oracle(oracle, params, topo, bins, frames, [t[k] for t, k in zip(tags, keep)])
    for rc, rr, k in zip(r_chk, r_ref, keep):
        assert not np.any(rc["uvengy"][~k]) and not np.any(rc["flceng"][~k])
        np.testing.assert_array_equal(rc["uvengy"][k], rr["uvengy"])
    for key in ("edens", "ecorr", "slnuv", "minuv", "maxuv", "engnorm", "engsmpl", "avslf", "voffset"):
        np.testing.assert_array_equal(a_chk[key], a_ref[key], err_msg=key)
    assert a_chk["engsmpl"] == sum(int(k.sum()) for k in keep)


def test_oracle_check_off_and_errors(oracle):
    params, topo, bins, frame, mass, host, solutes = _system()
    orc = oracle.Oracle(params, topo, bins)
    orc.set_aggregate(host, mass)
    orc.set_configuration_check(1, 0.0, 0.0)  # insposition 1: nothing checked
    pos, cell = frame(0)
    orc.frame(pos, cell)
    r = orc.placements(solutes)
    assert np.all(np.any(r["uvengy"] != 0, axis=1))
    orc.close()
    # slab checks need a periodic system (engproc.F90:1087)
    p = dict(params, boxshp=0, cltype=0, estype=1)
    orc = oracle.Oracle(p, topo, bins)
    orc.set_aggregate(host, mass)
    with pytest.raises(oracle.OracleError) as ei:
        orc.set_configuration_check(3, 0.0, 1.0)
    assert ei.value.code == oracle.E_ENG_SLB
    orc.set_configuration_check(2, 0.0, 1.0)  # the sphere check is allowed
    orc.close()


def test_oracle_fit_matches_lapack(oracle):
    """The oracle's best fit (a Jacobi eigensolver in place of dsyev) against numpy's LAPACK
    on random weighted point sets, and an exact rigid motion recovered."""
    from tests import insert_ref
    rng = np.random.default_rng(3)
    for n in (3, 6, 25):
        a = rng.normal(size=(n, 3)) * 3
        refa = rng.normal(size=(n, 3)) * 3
        w = rng.uniform(0.2, 2.0, n)
        if n > 4:
            w[0] = 0.0  # a masked atom (three weighted points at least: the fit is unique)
        b = rng.normal(size=(4, 3)) * 5
        np.testing.assert_allclose(oracle.fit_a_rotate_b(refa, a, w, b), insert_ref.horn_fit(refa, a, w, b),
                                   rtol=0, atol=1e-11)
        th = rng.uniform(0, 2 * np.pi)
        R = np.array([[1, 0, 0], [0, np.cos(th), -np.sin(th)], [0, np.sin(th), np.cos(th)]])
        moved = a @ R.T + rng.normal(size=3)
        np.testing.assert_allclose(oracle.fit_a_rotate_b(moved, a, w, a), moved, rtol=0, atol=1e-11)


# ---------------------------------------------------------------------------------- GPU
def _gpu(params, topo, bins, precision, check=None, batch=0):
    from ermod_gb300.engproc import EnergyRepresentation
    g = EnergyRepresentation(params, topo, bins, precision=precision, batch=batch)
    if check is not None:
        _configure(g, check)
    return g


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", CASES, ids=CASE_IDS)
def test_gpu_skip_matches_oracle(gpu_lib, oracle, precision, case):
    insposition = case["insposition"]
    params, topo, bins, frames, check, tags, keep = _setup(wgtslf=1, **case)
    r_orc, a_orc = _run_oracle(oracle, params, topo, bins, frames, tags, check)
    gpu = _gpu(params, topo, bins, precision, check, batch=4)  # placements span batches
    # two species: the waters (bin block 1) and the other solute molecules (block 2); each
    # placement's own solute has no energy
    n1 = int(bins["uvmax"][0])
    e1, e2 = bins["uvcrd"][:n1], bins["uvcrd"][n1:]
    nw = int(topo["nummol"]) - NSLT
    first = int(topo["nummol"]) - NSLT + 1
    ug1, uo1, ug2, uo2, u0 = [], [], [], [], []
    for (pos, cell), tg, k, ro in zip(frames, tags, keep, r_orc):
        gpu.frame(pos, cell)
        rg = gpu.placements(tg, want_uvengy=True, want_flceng=True)
        assert not np.any(rg["uvengy"][~k]) and not np.any(rg["flceng"][~k]), "rejected rows are zero"
        helpers.check_energies(rg["uvengy"][k], ro["uvengy"][k], precision, f"config check {insposition}")
        for p in np.nonzero(k)[0]:
            others = np.delete(np.arange(1 + nw, 1 + nw + NSLT), tg[p] - first)
            ug1.append(rg["uvengy"][p, 1:1 + nw])
            uo1.append(ro["uvengy"][p, 1:1 + nw])
            ug2.append(rg["uvengy"][p, others])
            uo2.append(ro["uvengy"][p, others])
            u0.append(ro["uvengy"][p, 0])
    ug1, uo1, ug2, uo2, u0 = (np.array(x) for x in (ug1, uo1, ug2, uo2, u0))
    rep = helpers.check_histograms(ug1, uo1, e1, precision, f"config check {insposition}")
    rep2 = helpers.check_histograms(ug2, uo2, e2, precision, f"config check {insposition}, solutes")
    rep["other_bin"] += rep2["other_bin"]
    ag = gpu.accum()
    gpu.close()
    assert ag["engsmpl"] == a_orc["engsmpl"] == len(u0)
    from ermod_gb300 import synth
    sol = synth.methanol_like()
    tol0 = helpers.self_tol(precision, sol)
    # voffset: the first accumulated placement's self energy (a rejected one comes first)
    np.testing.assert_allclose(ag["voffset"], a_orc["voffset"], rtol=0, atol=tol0)
    assert a_orc["voffset"] == u0[0]
    # solution-mode weights exp((u0 - voffset)/kT) (engproc.F90:772-796), NVT
    temp = params["temp"]
    wts = np.exp((u0 - u0[0]) / temp)
    rtol_w = helpers.weight_rtol(precision, sol, temp)
    np.testing.assert_allclose(ag["engnorm"], a_orc["engnorm"], rtol=max(rtol_w, 1e-12))
    if precision == "fp64" or rep["other_bin"] == 0:
        np.testing.assert_allclose(ag["edens"], a_orc["edens"], rtol=max(rtol_w, 1e-12), atol=0)
    b_ed, b_ec = helpers.weighted_bounds(None, wts, None, helpers.mixed_band(sol), rtol_w, corr=True,
                                         blocks=[(uo1, e1), (uo2, e2)])
    assert np.all(np.abs(ag["edens"] - a_orc["edens"]) <= b_ed + 1e-12 * np.abs(a_orc["edens"]))
    assert np.all(np.abs(ag["ecorr"] - a_orc["ecorr"]) <= b_ec + 1e-12 * np.abs(a_orc["ecorr"]))
    for sp in range(1, len(ag["minuv"])):
        np.testing.assert_allclose(ag["minuv"][sp], a_orc["minuv"][sp], atol=helpers.ENERGY_TOL[precision][0])
        np.testing.assert_allclose(ag["maxuv"][sp], a_orc["maxuv"][sp], atol=helpers.ENERGY_TOL[precision][0])
    np.testing.assert_allclose(ag["slnuv"], a_orc["slnuv"], rtol=max(rtol_w, 1e-9),
                               atol=topo["nummol"] * helpers.ENERGY_TOL[precision][0] * ag["engnorm"])


@pytest.mark.gpu
def test_gpu_slab_needs_periodic(gpu_lib):
    from ermod_gb300 import _lib
    params, topo, bins, frame, mass, host, solutes = _system()
    p = dict(params, boxshp=0, cltype=0, estype=1)
    g = _gpu(p, topo, bins, "fp64")
    g.set_aggregate(host, mass)
    with pytest.raises(_lib.ErmodError) as ei:
        g.set_configuration_check(4, 0.0, 1.0)
    assert ei.value.code == _lib.E_ENG_SLB
    g.set_configuration_check(2, 0.0, 1.0)
    g.close()
