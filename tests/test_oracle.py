"""The FP64 oracle pinned to the reference's golden vectors and to analytic checks (CPU).

Golden vectors: spline_test.F90:19-40 (the reference's only unit test).  Everything else
is analytic: the 3-D FFT against numpy, PME against a direct Ewald sum, the LJ switching
endpoints, the default energy-coordinate edges, the screening bisection.
"""
import math

import numpy as np
import pytest

# spline_test.F90:22-39 -- (order, x, M_order(x)), relative tolerance 1e-4 as there
GOLDEN_SPLINE = [
    (2, 0.0, 0.0), (2, 2.0, 0.0), (2, 1.0, 1.0), (2, 0.5, 0.5), (2, 1.5, 0.5),
    (6, 0.0, 0.0), (6, 6.0, 0.0), (6, 0.5, 2.604166666666667e-4), (6, 1.5, 6.171875000000000e-2),
    (6, 2.5, 0.438020833333333), (6, 3.5, 0.438020833333333), (6, 4.5, 6.171875000000000e-2),
    (6, 5.5, 2.604166666666667e-4),
]


@pytest.mark.parametrize("order,x,expect", GOLDEN_SPLINE)
def test_spline_golden(oracle, order, x, expect):
    got = oracle.spline_value(order, x)
    if expect == 0.0:
        assert got == 0.0
    else:
        assert abs(got - expect) <= 1e-4 * abs(expect)


def test_spline_partition_of_unity(oracle):
    for order in (4, 6, 8):
        for t in np.linspace(0.0, 0.999, 17):
            s = sum(oracle.spline_value(order, t + j) for j in range(order))
            assert abs(s - 1.0) < 1e-12  # the alternating sum loses a few digits at order 8


@pytest.mark.parametrize("shape", [(8, 6, 10), (32, 32, 32), (15, 12, 20), (7, 9, 14)])
def test_fft_matches_numpy(oracle, shape):
    rng = np.random.default_rng(1)
    g = rng.standard_normal(shape)
    a = oracle.fft_r2c_3d(g)
    b = np.fft.rfftn(g)
    assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()
    r = oracle.fft_c2r_3d(b, shape[2])
    rr = np.fft.irfftn(b, s=shape, axes=(0, 1, 2)) * np.prod(shape)
    assert np.abs(r - rr).max() <= 1e-13 * np.abs(rr).max()


def test_getscrn(oracle):
    beta = oracle.getscrn(1e-6, 12.0)
    assert abs(math.erfc(beta * 12.0) / 12.0 - 1e-6) < 1e-15
    from ermod_gb300 import setconf
    assert setconf.getscrn(1e-6, 12.0) == beta


def test_default_energy_coordinate(oracle):
    """pemax = 1396, region edges at the indices the construction fixes."""
    crd, pemax, pesoft = oracle.enginit_species(oracle.HIST_DEFAULT)
    assert (pemax, pesoft) == (1396, 1196)
    idx = [1, 397, 497, 697, 797, 1197, 1396]
    vals = [-20.02, -0.22, -0.02, 0.02, 0.22, 20.22, 1.0e11]
    for i, v in zip(idx, vals):
        assert abs(crd[i - 1] - v) <= 1e-12 * max(1.0, abs(v)), (i, crd[i - 1], v)
    assert np.all(np.diff(crd) > 0)


def test_product_setup_helpers_match_oracle(oracle):
    """The library's host helpers (enginit, LJ tables, charge scaling) == the oracle's."""
    from ermod_gb300 import setconf, synth
    for w in (synth.soln_small(), synth.refs_small(), synth.refs_large()):
        slt = w.params["slttype"]
        a = setconf.setparam_topology(w.species(), slttype=slt)
        b = oracle.setparam_topology(w.species(), slttype=slt)
        for k in a:
            np.testing.assert_array_equal(np.asarray(a[k]), np.asarray(b[k]), err_msg=k)
        ba = setconf.enginit_bins(a["numslv"])
        bb = oracle.enginit_bins(b["numslv"])
        for k in ba:
            np.testing.assert_array_equal(np.asarray(ba[k]), np.asarray(bb[k]), err_msg=k)


def test_lj_formats_and_combination(oracle):
    from ermod_gb300 import setconf
    sp = [dict(count=2, sluvid=0, charge=[0.1, -0.1], eps=[0.2, 0.3], len=[1.5, 1.7]),
          dict(count=1, sluvid=1, charge=[0.0, 0.0], eps=[0.2, 0.05], len=[1.5, 2.0])]
    for fmt in (0, 1, 2):
        for cmb in (0, 1):
            a = setconf.setparam_topology(sp, 1, ljformat=fmt, cmbrule=cmb)
            b = oracle.setparam_topology(sp, 1, ljformat=fmt, cmbrule=cmb)
            assert a["ljtype_max"] == b["ljtype_max"] == 3  # (1.5, 0.2) deduplicated
            np.testing.assert_allclose(a["ljene_mat"], b["ljene_mat"], rtol=1e-15)
            np.testing.assert_allclose(a["ljlensq_mat"], b["ljlensq_mat"], rtol=1e-15)


@pytest.mark.parametrize("sw", [0, 1, 2, 3])
def test_lj_switch_continuity(oracle, sw):
    """Each switch form is continuous at lwljcut and vanishes at upljcut."""
    p = oracle.OrcParams(slttype=1, estype=2, ljswitch=sw, splodr=4, ms1max=32, ms2max=32, ms3max=32,
                         elecut=12.0, lwljcut=10.0, upljcut=12.0, screen=0.34, temp=0.596, block_threshold=4.0)
    L = oracle.lib()
    eps, sg2 = 0.15, 3.15 ** 2
    lw2, up2 = 100.0, 144.0
    below = L.orc_pair_energy(p, eps, sg2, 0.0, lw2 * (1 - 1e-12))
    above = L.orc_pair_energy(p, eps, sg2, 0.0, lw2 * (1 + 1e-12))
    assert abs(below - above) < 1e-9
    assert abs(L.orc_pair_energy(p, eps, sg2, 0.0, up2)) < 1e-12
    assert L.orc_pair_energy(p, eps, sg2, 0.0, up2 * 1.0001) == 0.0


def test_pme_converges_to_direct_ewald(oracle):
    """PME reciprocal energies (spread, R2C, engfac, C2R, gather) -> direct Ewald sum."""
    from tests import helpers
    from ermod_gb300 import synth
    errs = []
    for K, order in [(32, 4), (48, 6), (64, 8)]:
        w = synth.Workload("t", "refs", 20.0, 250, synth.methanol_like(), synth._params(2, K, 0, 0), 9, 1, 4, 7)
        w.params["splodr"] = order
        topo, bins = helpers.build_inputs(w)
        orc = oracle.Oracle(w.params, topo, bins)
        pos, cell = w.frame(0)
        orc.frame(pos, cell)
        pl = w.placements(0, 1)
        rp, rself = orc.recip_parts(topo["nummol"], pl[0])
        de, dself = orc.direct_ewald(topo["nummol"], pl[0], mmax=14)
        errs.append(max(np.abs(rp - de).max(), abs(rself - dself)))
    assert errs[0] < 2e-3 and errs[1] < 2e-6 and errs[2] < 2e-9, errs


def test_histogram_normalisation_invariant(oracle):
    """slvfe.F90:495-512: sum of edens over a species = number of its molecules."""
    from ermod_gb300 import synth
    from tests import helpers
    w = synth.soln_small()
    topo, bins = helpers.build_inputs(w)
    orc = oracle.Oracle(w.params, topo, bins)
    for f in range(2):
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        orc.placements([topo["nummol"]])
    a = orc.accum()
    assert abs(a["edens"].sum() / a["engnorm"] - 1000.0) < 1e-9


def test_bin_errors(oracle):
    """eng_min (energy at or below the first edge) and eng_sft (solution mode)."""
    from ermod_gb300 import synth
    from tests import helpers
    w = synth.soln_small()
    hist = dict(oracle.HIST_DEFAULT)
    hist["ecdmin"] = -0.3  # first edge (-0.32) above the most negative energies
    topo, bins = helpers.build_inputs(w, hist)
    orc = oracle.Oracle(w.params, topo, bins)
    pos, cell = w.frame(0)
    orc.frame(pos, cell)
    r = orc.placements([topo["nummol"]], raise_on_error=False)
    assert r["status"] == oracle.E_ENG_MIN
    hist = dict(oracle.HIST_DEFAULT)
    hist["eccore"] = 0.1  # soft region ends below the most positive energies
    topo, bins = helpers.build_inputs(w, hist)
    orc = oracle.Oracle(w.params, topo, bins)
    orc.frame(pos, cell)
    assert orc.placements([topo["nummol"]], raise_on_error=False)["status"] == oracle.E_ENG_SFT


def test_pppm_converges_to_direct_ewald(oracle):
    """PPPM (cltype 3: the optimal influence function of recpcal_pppm_greenfunc in place
    of PME's engfac) -> direct Ewald sum, as the grid refines."""
    from tests import helpers
    from ermod_gb300 import synth
    errs = []
    for K, order in [(32, 4), (48, 6), (64, 8)]:
        w = synth.Workload("t", "refs", 20.0, 250, synth.methanol_like(), synth._params(2, K, 0, 0), 9, 1, 4, 7)
        w.params["splodr"] = order
        w.params["cltype"] = 3
        topo, bins = helpers.build_inputs(w)
        orc = oracle.Oracle(w.params, topo, bins)
        pos, cell = w.frame(0)
        orc.frame(pos, cell)
        pl = w.placements(0, 1)
        rp, rself = orc.recip_parts(topo["nummol"], pl[0])
        de, dself = orc.direct_ewald(topo["nummol"], pl[0], mmax=14)
        errs.append(max(np.abs(rp - de).max(), abs(rself - dself)))
    assert errs[0] < 1e-3 and errs[1] < 1e-6 and errs[2] < 1e-9, errs
