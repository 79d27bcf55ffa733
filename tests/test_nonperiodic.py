"""Non-periodic systems (boxshp 0): realcal_bare without minimum image and with an
infinite Coulomb cutoff (realcal.F90:155-281, reelcut = 1e50 at :170-178), no wrap in
realcal_prepare (:145), NVT and bare Coulomb only (setconf.F90:368-372), and no random or
slab insertion (insertion.F90:155,186).

CPU: the oracle against a numpy pair sum on a water droplet centred on the origin, and
the parameter checks of the oracle and of the C ABI.  GPU (marked): both precisions
against the oracle, histograms included, and the insertion / reach errors.
"""
import ctypes as C

import numpy as np
import pytest

from tests import helpers


def _droplet_inputs():
    from ermod_gb300 import synth
    w = synth.droplet()
    topo, bins = helpers.build_inputs(w)
    return w, topo, bins


def _pair_energies_numpy(w, topo, pos):
    """u_k = sum over solute x molecule-k site pairs of LJ (CHARMM potential switch,
    realcal.F90:218-236) + q q / r with no cutoff: the reference's realcal_bare for a
    non-periodic system, written independently of the oracle."""
    mbi = np.asarray(topo["mol_begin_index"]) - 1
    q = np.asarray(topo["charge"])
    lt = np.asarray(topo["ljtype"]) - 1
    eps_m = np.asarray(topo["ljene_mat"])
    sg2_m = np.asarray(topo["ljlensq_mat"])
    lw, up = w.params["lwljcut"], w.params["upljcut"]
    nummol = topo["nummol"]
    su = np.arange(mbi[nummol - 1], mbi[nummol])
    out = []
    for k in range(nummol - 1):
        sv = np.arange(mbi[k], mbi[k + 1])
        d = pos[su][:, None, :] - pos[sv][None, :, :]
        r2 = (d * d).sum(-1)
        r = np.sqrt(r2)
        eps = eps_m[lt[su][:, None], lt[sv][None, :]]
        sg2 = sg2_m[lt[su][:, None], lt[sv][None, :]]
        inv6 = (sg2 / r2) ** 3
        lj = 4.0 * eps * inv6 * (inv6 - 1.0)
        sw = (2.0 * r2 + up * up - 3.0 * lw * lw) * (r2 - up * up) ** 2 / (up * up - lw * lw) ** 3
        lj = np.where(r > lw, sw * lj, lj)
        lj = np.where(r > up, 0.0, lj)
        el = q[su][:, None] * q[sv][None, :] / r
        out.append((lj + el).sum())
    return np.array(out)


def test_oracle_droplet_matches_pair_sum(oracle):
    w, topo, bins = _droplet_inputs()
    orc = oracle.Oracle(w.params, topo, bins)
    for f in range(2):
        pos, cell = w.frame(f)
        assert np.all(cell == 0.0) and pos.min() < -10.0  # a zero cell and negative coordinates
        orc.frame(pos, cell)
        r = orc.placements([topo["nummol"]])
        ref = _pair_energies_numpy(w, topo, pos)
        # tagpt: the 300 waters, then the solute's own slot (0)
        np.testing.assert_allclose(r["uvengy"][0, 1:-1], ref, rtol=1e-12, atol=1e-12)
        assert r["uvengy"][0, -1] == 0.0
        assert r["uvengy"][0, 0] == 0.0  # realcal_self and residual_ene give nothing for bare Coulomb
        # beyond elecut the Coulomb term is still there (no cutoff without periodicity)
        far = np.linalg.norm(pos[0:3 * len(ref):3] - pos[-6], axis=1) > 12.5
        assert np.any(far) and np.all(np.abs(ref[far]) > 0.0)


def test_oracle_rejects_nonperiodic_pme_or_npt(oracle):
    w, topo, bins = _droplet_inputs()
    for bad in (dict(cltype=2), dict(estype=2)):
        p = dict(w.params)
        p.update(bad)
        with pytest.raises(oracle.OracleError):
            oracle.Oracle(p, topo, bins)


def test_abi_boxshp_checks_before_touching_a_device(gpu_lib):
    from ermod_gb300 import _lib
    p = _lib.Params()
    gpu_lib.ermod_default_params(C.byref(p))
    assert p.boxshp == 1
    ctx = C.c_void_p()
    for cltype, estype in ((2, 1), (0, 2), (3, 1)):
        bad = _lib.Params.from_buffer_copy(p)
        bad.boxshp, bad.cltype, bad.estype = 0, cltype, estype
        assert gpu_lib.ermod_create(C.byref(bad), 0, C.byref(ctx)) == _lib.E_SET_PRS
    bad = _lib.Params.from_buffer_copy(p)
    bad.boxshp = 2
    assert gpu_lib.ermod_create(C.byref(bad), 0, C.byref(ctx)) == _lib.E_PARAM


def test_abi_version_1_struct_is_read_without_boxshp(gpu_lib):
    """A version-1 caller's struct ends before boxshp: whatever follows it is not read
    (periodic system), so a PME context is not refused as set_prs."""
    from ermod_gb300 import _lib
    p = _lib.Params()
    gpu_lib.ermod_default_params(C.byref(p))
    p.abi_version = 1
    p.screen = 0.34
    p.boxshp = 0  # would be set_prs if it were read
    ctx = C.c_void_p()
    st = gpu_lib.ermod_create(C.byref(p), 0, C.byref(ctx))
    assert st != _lib.E_SET_PRS and st != _lib.E_PARAM
    if st == _lib.OK:
        gpu_lib.ermod_destroy(ctx)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_droplet_gpu_matches_oracle(gpu_lib, oracle, precision):
    from ermod_gb300.engproc import EnergyRepresentation
    w, topo, bins = _droplet_inputs()
    gpu = EnergyRepresentation(w.params, topo, bins, precision=precision)
    orc = oracle.Oracle(w.params, topo, bins)
    edges = np.asarray(bins["uvcrd"])
    for f in range(3):
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        ro = orc.placements([topo["nummol"]])
        gpu.frame(pos, cell)
        rg = gpu.placements([topo["nummol"]], want_uvengy=True)
        ug, uo = rg["uvengy"][0], ro["uvengy"][0]
        helpers.check_energies(ug, uo, precision, "droplet")
        helpers.check_histograms(ug[1:], uo[1:], edges, precision, "droplet")
    ag, ao = gpu.accum(), orc.accum()
    np.testing.assert_allclose(ag["engnorm"], ao["engnorm"], rtol=1e-12)
    np.testing.assert_allclose(ag["edens"].sum(), ao["edens"].sum(), rtol=1e-12)
    gpu.close()


@pytest.mark.gpu
def test_droplet_insertion_and_reach_errors(gpu_lib, oracle):
    """Random and slab insertion stop with ins_geo; a solute coordinate beyond the reach
    of the frame's fixed-point cube is reported by the device check (no fault)."""
    from ermod_gb300 import _lib
    from ermod_gb300.engproc import EnergyRepresentation
    from ermod_gb300 import synth
    w, topo, bins = _droplet_inputs()
    p = dict(w.params)
    p["slttype"] = 2  # reference-solvent mode: placements are given
    topo_r, bins_r = helpers.build_inputs(synth.Workload("d", "refs", w.box, w.nwater, w.solute, p, w.seed, 1, 4,
                                                         w.lattice_n, droplet=w.droplet))
    gpu = EnergyRepresentation(p, topo_r, bins_r, precision="mixed")
    pos, cell = w.frame(0)
    gpu.frame(pos, cell)
    sl = w.solute["xyz"] - w.solute["xyz"].mean(0)
    for mode in (0, 3, 4):
        with pytest.raises(_lib.ErmodError) as ei:
            gpu.generate_placements(4, sl, w.solute["mass"], insposition=mode, lwreg=0.0, upreg=1.0)
        assert ei.value.code == _lib.E_INS_GEO
    sol, _ = gpu.generate_placements(8, sl, w.solute["mass"], insposition=2, lwreg=0.0, upreg=1.5)
    pl = sol.cpu().numpy()
    tag = np.full(len(pl), topo_r["nummol"], np.int32)
    rg = gpu.placements(tag, pl, want_uvengy=True)
    orc = oracle.Oracle(p, topo_r, bins_r)
    orc.frame(pos, cell)
    ro = orc.placements(tag, pl)
    helpers.check_energies(rg["uvengy"], ro["uvengy"], "mixed", "droplet insertions")
    far = pl.copy()
    far[0] += 1.0e4
    with pytest.raises(_lib.ErmodError) as ei:
        gpu.placements(tag[:1], far[:1], want_uvengy=True)
    assert ei.value.code == _lib.E_DEVICE
    gpu.close()
