"""The parity checks themselves (CPU): they pass on energies within the stated band and
fail when a molecule away from every bin edge lands in another bin, or when a weighted
accumulator moves by more than its near-edge molecules allow.  The energies are the
oracle's; the mistakes are planted in a copy of them, on the CPU."""
import numpy as np
import pytest

from tests import helpers


@pytest.fixture(scope="module")
def energies(oracle):
    w = helpers.small_refs()
    topo, bins = helpers.build_inputs(w)
    orc = oracle.Oracle(w.params, topo, bins)
    pos, cell = w.frame(0)
    orc.frame(pos, cell)
    pl = w.placements(0, 12)
    u = orc.placements(np.full(len(pl), topo["nummol"], np.int32), pl)["uvengy"]
    orc.close()
    return u, np.asarray(bins["uvcrd"]), w


def _near_edge_shift(uo, edges, band):
    """A copy of uo with every molecule within the band of an edge moved across it."""
    ug = uo.copy()
    for p in range(len(ug)):
        b = helpers.bin_index(uo[p], edges)
        up = (b + 1 < len(edges)) & (np.abs(uo[p] - edges[np.minimum(b + 1, len(edges) - 1)]) <= band)
        ug[p, up] = edges[b[up] + 1] + 0.5 * band  # just above the upper edge: bin b + 1
    return ug


def test_band_flips_pass_and_are_counted(energies):
    u, edges, _ = energies
    uo = u[:, 1:]
    band = helpers.MIXED_BAND
    ug = _near_edge_shift(uo, edges, band)
    rep = helpers.check_histograms(ug, uo, edges, "mixed", "planted near-edge flips")
    assert rep["other_bin"] > 0 and rep["other_bin"] <= rep["near_edge_band"]


def test_far_flip_fails(energies):
    u, edges, _ = energies
    uo = u[:, 1:]
    d = helpers.edge_distance(uo[0], edges)
    k = int(np.argmax(np.where(np.abs(uo[0]) < 20, d, -1.0)))  # a molecule far from any edge
    ug = uo.copy()
    b = helpers.bin_index(uo[0, k:k + 1], edges)[0]
    ug[0, k] = edges[b + 1] + 0.5 * (edges[b + 2] - edges[b + 1])  # the middle of the next bin
    with pytest.raises(AssertionError):
        helpers.check_histograms(ug, uo, edges, "mixed", "planted far flip")


def test_energy_bound_fails_beyond_band(energies):
    u, _, _ = energies
    ug = u.copy()
    ug[3, 17] += 2 * helpers.MIXED_BAND
    with pytest.raises(AssertionError):
        helpers.check_energies(ug, u, "mixed")
    helpers.check_energies(u + 0.5 * helpers.MIXED_BAND, u, "mixed")


def test_weighted_bounds(energies):
    u, edges, w = energies
    uo = u[:, 1:]
    wts = np.exp(-(u[:, 0] - u[0, 0]) / w.params["temp"])
    band = helpers.MIXED_BAND
    b_ed, b_ec = helpers.weighted_bounds(uo, wts, edges, band, 0.0, corr=True)

    def accum(uu):
        H = np.stack([helpers.histogram(x, edges) for x in uu]).astype(float)
        return (wts[:, None] * H).sum(0), (wts[:, None] * H).T @ H

    ed0, ec0 = accum(uo)
    ed1, ec1 = accum(_near_edge_shift(uo, edges, band))
    assert np.any(ed1 != ed0)
    assert np.all(np.abs(ed1 - ed0) <= b_ed * (1 + 1e-12))
    assert np.all(np.abs(ec1 - ec0) <= b_ec * (1 + 1e-12) + 1e-12)
    # a molecule far from every edge moved: beyond the bounds
    far = uo.copy()
    d = helpers.edge_distance(uo[0], edges)
    k = int(np.argmax(np.where(np.abs(uo[0]) < 20, d, -1.0)))
    b = helpers.bin_index(uo[0, k:k + 1], edges)[0]
    far[0, k] = edges[b + 1] + 0.5 * (edges[b + 2] - edges[b + 1])
    ed2, _ = accum(far)
    assert np.any(np.abs(ed2 - ed0) > b_ed * (1 + 1e-12))
