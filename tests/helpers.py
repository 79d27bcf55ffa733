"""Shared set-up and tolerances of the parity tests: one workload, the oracle and the GPU engine.

Per-molecule energies, kcal/mol, against the FP64 oracle:
  |u_gpu - u_oracle| <= atol + rtol |u_oracle|          (ENERGY_TOL)
  FP64 path    atol 1e-9, rtol 1e-11: summation order only.
  mixed path   atol MIXED_BAND, rtol 1e-13.  The FP32 quantities of a molecule's energy
               are its reciprocal site terms q phi (up to ~100 kcal/mol for a site next to
               the solute, each carrying the FP32 rounding of the potential grid, of the
               transforms and of the 64-point gather: about 2^-24 x sqrt(64) relative) and
               its real-space pair terms below 8 kcal/mol (larger ones run in FP64); the
               terms are summed as float-float numbers, so the sums add no rounding of
               their own.  MIXED_BAND bounds the first two with a margin of about two over
               the largest error seen (1.2e-5 for a site 2.5 A from a 12-site solute);
               rtol covers the float-float totals (2^-48) of overlapping pairs, whose FP64
               terms reach 1e10 kcal/mol.
Histograms: a molecule may take the neighbouring bin only when its oracle energy lies
within MIXED_BAND of a bin edge; every other molecule is binned exactly as the oracle bins
it.  The tests count the molecules within 1e-6 and within MIXED_BAND of an edge and the
molecules binned elsewhere, and print them.
Large, strongly charged solutes: mixed_band(solute) grows the band as sqrt(sum|q| / 3 e).
Solute self energies (they set the weights engnmfc = exp(-(u0 - voffset)/kT) V): FP64
1e-9; mixed self_tol(solute) = 2e-6 kcal/mol x sqrt(max(n, 12) / 12) x max(1, sum q^2 / 1.1)
for an n-site solute.  The B-spline weights and 1-D structure factors are FP64, rounded
once to FP32; the spectrum S(k) = sum_s q_s b1 b2 b3 is summed over the sites in FP32,
whose independent roundings grow as sqrt(n) and with the charges; the engfac |S|^2 terms
are summed per tile in FP32 and across tiles as float-float numbers.  Largest errors seen:
3.7e-7 (12 sites), 4.4e-6 (40 sites, sum q^2 = 3.6 e^2), 3.9e-6 (256 sites).
"""
import numpy as np

from ermod_gb300 import setconf, synth

MIXED_BAND = 3e-5
ENERGY_TOL = {"fp64": (1e-9, 1e-11), "mixed": (MIXED_BAND, 1e-13)}


def mixed_band(solute=None):
    """The mixed path's per-molecule bound for a solute: MIXED_BAND, grown as the square root
    of the solute's summed absolute charge beyond 3 e (the potential next to a large,
    strongly charged solute is larger, and so are the FP32 roundings of q phi; measured:
    1.3e-5 kcal/mol at 1.4 e and 2.9 e, 2.4e-5 at 9.6 e)."""
    if solute is None:
        return MIXED_BAND
    q1 = float(np.sum(np.abs(solute["charge"])))
    return MIXED_BAND * max(1.0, np.sqrt(q1 / 3.0))


def self_tol(precision, solute):
    """Tolerance of the solute self energy u0 (kcal/mol) of a solute (a dict with its site
    charges): 2e-6 kcal/mol, grown as sqrt(n / 12) for n > 12 sites (the spectrum sums n FP32
    products) and in proportion to the summed squared charges beyond 1.1 e^2."""
    if precision == "fp64":
        return 1e-9
    q = np.asarray(solute["charge"], float)
    return 2e-6 * np.sqrt(max(len(q), 12) / 12.0) * max(1.0, float(np.sum(q * q)) / 1.1)


def weight_rtol(precision, solute, temp):
    """Relative tolerance of the weights exp(-(u0 - voffset)/kT): u0 and voffset each
    within self_tol."""
    return 1e-10 if precision == "fp64" else 2 * self_tol(precision, solute) / temp + 1e-12


def small_refs(nwater=600, box=26.0, K=32, seed=21, corrcal=1, wgtslf=1, solute=None, lattice=9):
    sol = synth.methanol_like() if solute is None else solute
    return synth.Workload("refs_test", "refs", box, nwater, sol, synth._params(2, K, corrcal=corrcal, wgtslf=wgtslf),
                          seed, 1, 64, lattice)


def build_inputs(w, hist=None):
    topo = setconf.setparam_topology(w.species(), slttype=w.params["slttype"])
    bins = setconf.enginit_bins(topo["numslv"], hist)
    return topo, bins


def edge_distance(u, edges):
    """Distance of each u to the nearest bin edge."""
    idx = np.searchsorted(edges, u)
    lo = np.abs(u - edges[np.clip(idx - 1, 0, len(edges) - 1)])
    hi = np.abs(u - edges[np.clip(idx, 0, len(edges) - 1)])
    return np.minimum(lo, hi)


def near_edge(u, edges, tol):
    """True where u lies within tol of a bin edge."""
    return edge_distance(u, edges) <= tol


def bin_index(u, edges):
    """getiduv's bin (0-based): edges[k-1] < u <= edges[k]; the last bin is open above."""
    return np.searchsorted(edges, u, side="left") - 1


def histogram(u, edges):
    """insdst of one placement: bin k (1-based) <=> edges[k-1] < u <= edges[k]; last bin open."""
    return np.bincount(bin_index(u, edges), minlength=len(edges))


def check_energies(u_gpu, u_orc, precision, label="", band=None):
    """Every molecule's energy within ENERGY_TOL (mixed: atol = band when given); returns
    the largest errors (all, |u| < 20)."""
    atol, rtol = ENERGY_TOL[precision]
    if precision == "mixed" and band is not None:
        atol = band
    err = np.abs(u_gpu - u_orc)
    bound = atol + rtol * np.abs(u_orc)
    worst = int(np.argmax(err - bound))
    assert np.all(err <= bound), \
        f"{label} {precision}: max err {err.flat[worst]:.3e} at {worst} (u={u_orc.flat[worst]:.6f})"
    soft = np.abs(u_orc) < 20.0
    return float(err.max()), float(err[soft].max()) if np.any(soft) else 0.0


def check_histograms(u_gpu, u_orc, edges, precision, label="", band=None):
    """Per placement (rows of u): every molecule farther than the band from a bin edge is
    binned as the oracle bins it; the molecules near an edge and those binned elsewhere are
    counted (and printed).  FP64: no band beyond the FP64 energy tolerance."""
    if band is None:
        band = MIXED_BAND if precision == "mixed" else 1e-9
    u_gpu, u_orc = np.atleast_2d(u_gpu), np.atleast_2d(u_orc)
    n6 = nb = other = 0
    for ug, uo in zip(u_gpu, u_orc):
        d = edge_distance(uo, edges)
        near = d <= band
        bg, bo = bin_index(ug, edges), bin_index(uo, edges)
        moved = bg != bo
        assert not np.any(moved & ~near), \
            f"{label}: molecules farther than {band:g} from an edge binned elsewhere: {np.flatnonzero(moved & ~near)[:8]}"
        n6 += int(np.count_nonzero(d <= 1e-6))
        nb += int(np.count_nonzero(near))
        other += int(np.count_nonzero(moved))
        np.testing.assert_array_equal(np.bincount(bg[~near], minlength=len(edges)),
                                      np.bincount(bo[~near], minlength=len(edges)))
    assert other <= nb
    rep = dict(molecules=int(u_orc.size), near_edge_1e6=n6, near_edge_band=nb, band=band, other_bin=other)
    print(f"[parity] {label} {precision}: {rep}")
    return rep


def _counts_and_movers(u_orc, edges, band):
    """Per placement: the oracle's histogram H and, bin by bin, the molecules M within the
    band of one of the bin's edges (counted in the bin and in the neighbour across it)."""
    E = len(edges)
    H = np.stack([histogram(u, edges) for u in np.atleast_2d(u_orc)]).astype(float)
    M = np.zeros_like(H)
    for p, u in enumerate(np.atleast_2d(u_orc)):
        b = bin_index(u, edges)  # edges[b] < u <= edges[b + 1]
        up = (b + 1 < E) & (np.abs(u - edges[np.minimum(b + 1, E - 1)]) <= band)  # may move to b + 1
        dn = (b >= 1) & (np.abs(u - edges[np.clip(b, 0, E - 1)]) <= band)  # may move to b - 1
        for mask, tgt in ((up, b), (up, b + 1), (dn, b), (dn, b - 1)):
            np.add.at(M[p], tgt[mask], 1.0)
    return H, M


def weighted_bounds(u_orc, weights, edges, band, rtol_w, corr=False, blocks=None):
    """Bin-by-bin bounds on |edens_gpu - edens_orc| (and ecorr) of a weighted accumulation:
    rtol_w of the oracle's value for the weights' relative error, plus, per placement, its
    weight times the molecules within the band of either edge of the bin (each may sit in
    the neighbouring bin on the GPU).  Several solvent species: blocks = [(u_orc of the
    species' molecules, the species' edges), ...] in bin-block order (u_orc, edges unused)."""
    if blocks is None:
        blocks = [(u_orc, edges)]
    parts = [_counts_and_movers(u, e, band) for u, e in blocks]
    H = np.concatenate([h for h, _ in parts], axis=1)
    M = np.concatenate([m for _, m in parts], axis=1)
    w = np.asarray(weights, float)
    ed = (w[:, None] * H).sum(0)
    g = 1.0 + rtol_w  # a moved molecule carries the GPU's weight
    bound_ed = rtol_w * ed + g * (w[:, None] * M).sum(0)
    if not corr:
        return bound_ed, None
    wH, wM = w[:, None] * H, w[:, None] * M
    ec = wH.T @ H
    bound_ec = rtol_w * ec + g * (wM.T @ (H + M) + wH.T @ M)
    return bound_ed, bound_ec
