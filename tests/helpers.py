"""Shared set-up for the parity tests: one workload, the oracle and the GPU engine."""
import numpy as np

from ermod_gb300 import setconf, synth


def small_refs(nwater=600, box=26.0, K=32, seed=21, corrcal=1, wgtslf=1, solute=None, lattice=9):
    sol = synth.methanol_like() if solute is None else solute
    return synth.Workload("refs_test", "refs", box, nwater, sol, synth._params(2, K, corrcal=corrcal, wgtslf=wgtslf),
                          seed, 1, 64, lattice)


def build_inputs(w, hist=None):
    topo = setconf.setparam_topology(w.species(), slttype=w.params["slttype"])
    bins = setconf.enginit_bins(topo["numslv"], hist)
    return topo, bins


def near_edge(u, edges, tol):
    """True where u lies within tol of a bin edge."""
    idx = np.searchsorted(edges, u)
    lo = np.abs(u - edges[np.clip(idx - 1, 0, len(edges) - 1)])
    hi = np.abs(u - edges[np.clip(idx, 0, len(edges) - 1)])
    return np.minimum(lo, hi) <= tol


def histogram(u, edges):
    """insdst of one placement: bin k (1-based) <=> edges[k-1] < u <= edges[k]; last bin open."""
    ret = np.searchsorted(edges, u, side="left")  # number of edges < u
    return np.bincount(ret - 1, minlength=len(edges))
