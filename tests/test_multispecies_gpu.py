"""Two solvent species (water and a methanol-like cosolvent): per-species bin offsets,
uvspec, flceng, minuv/maxuv, slnuv and the edens blocks of each species, in
reference-solvent mode with ecorr, and in solution mode.

CPU: the oracle's edens blocks sum to each species' molecule count (slvfe's
normalisation, slvfe.F90:495-512).  GPU (marked): both precisions against the oracle.
"""
import numpy as np
import pytest

from tests import helpers


def _mixture(mode, seed=31, nwater=420, nmeoh=40, box=26.0, K=32):
    """(species, frames(i), placements(i, n), params) of a water + cosolvent box."""
    from ermod_gb300 import insertion, synth
    meoh = synth.methanol_like()
    rng = np.random.default_rng((seed, 3))
    sol = synth.random_solute(rng, 8)
    n = 9
    g = (np.arange(n) + 0.5) * (box / n)
    pts = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    if mode == "soln":
        pts = pts[np.linalg.norm(pts - box / 2, axis=1) > 5.0]
    pick = rng.choice(len(pts), nwater + nmeoh, replace=False)
    lat_w, lat_m = pts[pick[:nwater]], pts[pick[nwater:]]
    species = [dict(count=nwater, sluvid=0, charge=synth.WATER_CHARGE, eps=synth.WATER_EPS, len=synth.WATER_SIG),
               dict(count=nmeoh, sluvid=0, charge=meoh["charge"], eps=meoh["eps"], len=meoh["sig"]),
               dict(count=1, sluvid=1 if mode == "soln" else 2, charge=sol["charge"], eps=sol["eps"],
                    len=sol["sig"])]
    params = synth._params(1 if mode == "soln" else 2, K, corrcal=0 if mode == "soln" else 1, wgtslf=1)
    cell = np.diag([box] * 3)

    def place(body, mass, centres, r):
        body = body - insertion.center_of_mass(body, mass)
        q = insertion.random_quaternions(r, len(centres))
        return (insertion.quat_rotate(q, np.broadcast_to(body, (len(centres),) + body.shape))
                + centres[:, None, :]).reshape(-1, 3)

    def frame(i):
        r = np.random.default_rng((seed, 100 + i))
        w = place(synth.water_body(), synth.WATER_MASS, lat_w + r.uniform(-0.3, 0.3, lat_w.shape), r)
        m = place(meoh["xyz"], meoh["mass"], lat_m + r.uniform(-0.3, 0.3, lat_m.shape), r)
        s = sol["xyz"] - insertion.center_of_mass(sol["xyz"], sol["mass"]) + box / 2
        return np.ascontiguousarray(np.concatenate([w, m, s])), cell

    def placements(i, k):
        return insertion.random_placements(np.random.default_rng((seed, 900 + i)), sol["xyz"], sol["mass"], cell, k)

    return species, frame, placements, params


def _inputs(mode):
    from ermod_gb300 import setconf
    species, frame, placements, params = _mixture(mode)
    topo = setconf.setparam_topology(species, slttype=params["slttype"])
    assert topo["numslv"] == 2
    bins = setconf.enginit_bins(topo["numslv"])
    return species, frame, placements, params, topo, bins


def test_oracle_edens_blocks_count_each_species(oracle):
    species, frame, placements, params, topo, bins = _inputs("refs")
    orc = oracle.Oracle(params, topo, bins)
    pos, cell = frame(0)
    orc.frame(pos, cell)
    pl = placements(0, 6)
    orc.placements(np.full(len(pl), topo["nummol"], np.int32), pl)
    a = orc.accum()
    n1 = int(bins["uvmax"][0])
    # edens / engnorm per species = the number of molecules of that species
    assert abs(a["edens"][:n1].sum() / a["engnorm"] - species[0]["count"]) < 1e-9
    assert abs(a["edens"][n1:].sum() / a["engnorm"] - species[1]["count"]) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("mode", ["refs", "soln"])
def test_two_species_match_oracle(gpu_lib, oracle, precision, mode):
    from ermod_gb300.engproc import EnergyRepresentation
    species, frame, placements, params, topo, bins = _inputs(mode)
    gpu = EnergyRepresentation(params, topo, bins, precision=precision)
    orc = oracle.Oracle(params, topo, bins)
    n1 = int(bins["uvmax"][0])
    nw, nm = 420, 40  # columns of the waters, then of the cosolvent molecules
    uo_all = []
    for f in range(2):
        pos, cell = frame(f)
        orc.frame(pos, cell)
        gpu.frame(pos, cell)
        if mode == "refs":
            pl = placements(f, 20)
            tag = np.full(len(pl), topo["nummol"], np.int32)
            ro, rg = orc.placements(tag, pl), gpu.placements(tag, pl, want_uvengy=True, want_flceng=True)
        else:
            tag = [topo["nummol"]]
            ro, rg = orc.placements(tag), gpu.placements(tag, want_uvengy=True, want_flceng=True)
        ug, uo = rg["uvengy"][:, 1:], ro["uvengy"][:, 1:]
        helpers.check_energies(rg["uvengy"], ro["uvengy"], precision, f"two species {mode}")
        for cols, edges in ((slice(0, nw), bins["uvcrd"][:n1]), (slice(nw, nw + nm), bins["uvcrd"][n1:])):
            helpers.check_histograms(ug[:, cols], uo[:, cols], edges, precision, f"two species {mode}")
        # flceng: per species sums of the molecules' energies
        atol = helpers.ENERGY_TOL[precision][0] * nw
        np.testing.assert_allclose(rg["flceng"], ro["flceng"], rtol=helpers.ENERGY_TOL[precision][1], atol=atol)
        uo_all.append(ro["uvengy"])
    ag, ao = gpu.accum(), orc.accum()
    # wgtslf = 1: the weights follow the solute self energy (solution mode: exp(+(u0 - voffset)/kT))
    rtol_w = helpers.weight_rtol(precision, dict(charge=species[2]["charge"]), params["temp"])
    np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=rtol_w)
    for blk in (slice(0, n1), slice(n1, None)):  # the species blocks of edens
        np.testing.assert_allclose(ag["edens"][blk].sum(), ao["edens"][blk].sum(), rtol=rtol_w)
    if precision == "fp64":
        np.testing.assert_allclose(ag["edens"], ao["edens"], rtol=1e-10, atol=1e-12 * ao["engnorm"])
    for key in ("minuv", "maxuv"):
        np.testing.assert_allclose(ag[key], ao[key], rtol=helpers.ENERGY_TOL[precision][1],
                                   atol=helpers.ENERGY_TOL[precision][0])
    if mode == "soln":
        np.testing.assert_allclose(ag["slnuv"], ao["slnuv"], rtol=rtol_w, atol=atol * ao["engnorm"])
    gpu.close()
