"""Adjoint mode on the GPU (marked gpu): bin-resolved d u / d theta for every solute
site's charge, LJ epsilon and LJ sigma.

The GPU sums are compared, bin by bin, with the FP64 oracle's per-molecule analytic
derivatives and with FP64 central finite differences (step 1e-4 relative) of the
oracle's energies, both binned by the GPU's own energies.  Tolerance (the stated
target): 1e-3 of the bin's summed magnitude sum_k |d u_k / d theta|, with a floor of
1e-6 of the parameter's largest bin magnitude for bins whose derivatives nearly cancel
(FP32 terms of a molecule are about 1e-7 of their own size apart).
"""
import numpy as np
import pytest

from ermod_gb300 import setconf, synth

pytestmark = pytest.mark.gpu

NSITE = 6


def _system(ljswitch):
    rng = np.random.default_rng(31)
    sol = synth.random_solute(rng, NSITE)
    w = synth.Workload("adj_gpu", "soln", 24.0, 420, sol, synth._params(1, 24, corrcal=0, wgtslf=0), 17, 3, 1, 8,
                       cavity=4.5)
    w.params["ljswitch"] = ljswitch
    w.params["estype"] = 1  # unit weights: the bin weights are molecule counts
    w.params["lwljcut"], w.params["upljcut"], w.params["elecut"] = 8.0, 10.0, 10.0
    return w


def _topology(w, sol):
    sp = w.species()
    sp[1] = dict(sp[1], charge=sol["charge"], eps=sol["eps"], len=sol["sig"])
    topo = setconf.setparam_topology(sp, slttype=1)
    return topo, setconf.enginit_bins(topo["numslv"])


def _bins(u, edges):
    return np.searchsorted(edges, u, side="left") - 1


def _run_gpu(w, topo, bins, frames):
    from ermod_gb300.engproc import EnergyRepresentation
    gpu = EnergyRepresentation(w.params, topo, bins, precision="mixed")
    gpu.adjoint_enable()
    tag = topo["nummol"]
    us = []
    for f in frames:
        pos, cell = w.frame(f)
        gpu.frame(pos, cell)
        us.append(gpu.placements([tag], want_uvengy=True)["uvengy"][0, 1:].copy())
    g, wt = gpu.adjoint_get()
    gpu.close()
    return g, wt, us


def _check(g, ref, mag):
    err = np.abs(g - ref)
    bound = 1e-3 * mag + 1e-6 * mag.max(axis=1, keepdims=True) + 1e-12
    worst = np.unravel_index(np.argmax(err - bound), err.shape)
    assert np.all(err <= bound), (worst, float(err[worst]), float(ref[worst]), float(mag[worst]))


@pytest.mark.parametrize("ljswitch", [0, 2])
def test_adjoint_matches_oracle_gradient(gpu_lib, oracle, ljswitch):
    w = _system(ljswitch)
    sol = w.solute
    topo, bins = _topology(w, sol)
    frames = [0, 1, 2]
    g, wt, us = _run_gpu(w, topo, bins, frames)
    orc = oracle.Oracle(w.params, topo, bins)
    tag = topo["nummol"]
    edges = bins["uvcrd"]
    E, P = len(edges), 3 * NSITE
    ref = np.zeros((P, E))
    mag = np.zeros((P, E))
    cnt = np.zeros(E)
    for f, u in zip(frames, us):
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        du = orc.adjoint(tag)
        keep = np.ones(len(u), bool)
        keep[-1] = False  # the solute itself (last in tagpt order)
        b = _bins(u[keep], edges)
        np.add.at(ref.T, b, du[keep])
        np.add.at(mag.T, b, np.abs(du[keep]))
        np.add.at(cnt, b, 1.0)
    assert g.shape == (P, E)
    np.testing.assert_array_equal(wt, cnt)
    _check(g, ref, mag)


def test_adjoint_matches_central_differences(gpu_lib, oracle):
    w = _system(0)
    base = {k: (np.array(v, dtype=float) if k != "xyz" else v) for k, v in w.solute.items()}
    topo, bins = _topology(w, base)
    frames = [0, 1]
    g, wt, us = _run_gpu(w, topo, bins, frames)
    edges = bins["uvcrd"]
    tag = topo["nummol"]

    def energies(sol, f):
        t, bn = _topology(w, sol)
        orc = oracle.Oracle(w.params, t, bn)
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        return orc.placements([tag])["uvengy"][0, 1:]

    for s, col, key in ((0, 0, "charge"), (1, 1, "eps"), (2, 2, "sig"), (4, 0, "charge"), (5, 2, "sig")):
        p = 3 * s + col
        ref = np.zeros(len(edges))
        mag = np.zeros(len(edges))
        step = 1e-4 * abs(base[key][s])
        for f, u in zip(frames, us):
            up = dict(base, **{key: base[key].copy()})
            dn = dict(base, **{key: base[key].copy()})
            up[key][s] += step
            dn[key][s] -= step
            fd = (energies(up, f) - energies(dn, f)) / (2 * step)
            if key == "charge":
                fd = fd / setconf.CHARGE_SCALE  # per topology charge unit, as the adjoint reports
            keep = np.ones(len(u), bool)
            keep[-1] = False
            b = _bins(u[keep], edges)
            np.add.at(ref, b, fd[keep])
            np.add.at(mag, b, np.abs(fd[keep]))
        _check(g[p][None, :], ref[None, :], mag[None, :])


def test_adjoint_full_size_against_oracle_gradient(gpu_lib, oracle):
    """The adjoint workload at its own size: 8,000 waters in a 62 A box, a 16-site solute
    (48 parameters), PME 64^3, two frames; the oracle's FP64 gradient binned by the GPU's
    energies."""
    w = synth.soln_adjoint(frames=2)
    assert w.nwater == 8000 and len(w.solute["charge"]) == 16 and w.params["ms1max"] == 64
    topo = setconf.setparam_topology(w.species(), slttype=1)
    bins = setconf.enginit_bins(topo["numslv"])
    frames = [0, 1]
    g, wt, us = _run_gpu(w, topo, bins, frames)
    orc = oracle.Oracle(w.params, topo, bins)
    tag = topo["nummol"]
    edges = bins["uvcrd"]
    E, P = len(edges), 3 * 16
    ref = np.zeros((P, E))
    mag = np.zeros((P, E))
    cnt = np.zeros(E)
    for f, u in zip(frames, us):
        pos, cell = w.frame(f)
        orc.frame(pos, cell)
        du = orc.adjoint(tag)
        keep = np.ones(len(u), bool)
        keep[-1] = False
        b = _bins(u[keep], edges)
        np.add.at(ref.T, b, du[keep])
        np.add.at(mag.T, b, np.abs(du[keep]))
        np.add.at(cnt, b, 1.0)
    assert g.shape == (P, E)
    # NPT: every molecule's weight is the same volume factor C
    C = wt.sum() / cnt.sum()
    np.testing.assert_allclose(wt, cnt * C, rtol=1e-12)
    _check(g / C, ref, mag)
