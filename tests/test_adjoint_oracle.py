"""The FP64 oracle's analytic solute-parameter derivatives against central finite
differences of the oracle's own energies (CPU).

Each parameter theta (a solute site's charge, LJ epsilon or LJ sigma) is moved by
+-1e-4 relative, the topology (LJ tables included) is rebuilt, and the per-molecule
energies are differenced.  Every LJ switching form is covered.
"""
import numpy as np
import pytest

from ermod_gb300 import setconf, synth


def _system(ljswitch, cmbrule=0):
    rng = np.random.default_rng(31)
    sol = synth.random_solute(rng, 5)
    w = synth.Workload("adj_test", "soln", 24.0, 420, sol, synth._params(1, 24, corrcal=0, wgtslf=0), 17, 1, 1, 8,
                       cavity=4.5)
    w.params["ljswitch"] = ljswitch
    # solvent close enough to the solute for every LJ region to be populated
    w.params["lwljcut"], w.params["upljcut"], w.params["elecut"] = 8.0, 10.0, 10.0
    return w


def _energies(w, sol, cmbrule):
    from oracle import oracle as O
    sp = w.species()
    sp[1] = dict(sp[1], charge=sol["charge"], eps=sol["eps"], len=sol["sig"])
    topo = setconf.setparam_topology(sp, slttype=1, cmbrule=cmbrule)
    bins = setconf.enginit_bins(topo["numslv"])
    orc = O.Oracle(w.params, topo, bins)
    pos, cell = w.frame(0)
    orc.frame(pos, cell)
    tag = topo["nummol"]
    u = orc.placements([tag])["uvengy"][0, 1:]
    return orc, tag, u


@pytest.mark.parametrize("ljswitch,cmbrule", [(0, 0), (1, 0), (2, 1), (3, 0)])
def test_oracle_adjoint_matches_central_differences(oracle, ljswitch, cmbrule):
    w = _system(ljswitch)
    sol = {k: np.array(v, dtype=float) if k != "xyz" else v for k, v in w.solute.items()}
    orc, tag, u0 = _energies(w, sol, cmbrule)
    grad = orc.adjoint(tag, cmbrule=cmbrule)
    assert grad.shape == (orc.slvmax, 15)
    scale = setconf.CHARGE_SCALE
    h = 1e-4
    for s in range(5):
        for col, key in enumerate(("charge", "eps", "sig")):
            up, dn = dict(sol), dict(sol)
            step = h * abs(sol[key][s])
            up[key] = sol[key].copy()
            dn[key] = sol[key].copy()
            up[key][s] += step
            dn[key][s] -= step
            fd = (_energies(w, up, cmbrule)[2] - _energies(w, dn, cmbrule)[2]) / (2 * step)
            if key == "charge":
                fd = fd / scale  # the analytic derivative is per topology charge unit
            an = grad[:, 3 * s + col]
            err = np.abs(an - fd)
            bound = 1e-6 * np.abs(fd).max() + 1e-5 * np.abs(fd)
            assert np.all(err <= bound), (ljswitch, s, key, float(err.max()), float(np.abs(fd).max()))
