"""The mixed path bins an FP32 molecule total u against the FP64 edges (getiduv /
binsearch, engproc.F90:927-1020) with 32-bit keys: u against the edges rounded down to
floats.  For a float u and a double e, u <= e exactly when u <= rd(e), the largest float
not above e, so the count of edges below u is the same.  This checks that rule (the one
the finish kernel uses) on edges of the default energy coordinate, on edges a float
spacing apart, on signed zeros and beyond the float range (CPU, numpy)."""
import numpy as np

from ermod_gb300 import setconf


def _rd(edges):
    with np.errstate(over="ignore"):  # beyond the float range: +-inf, then rounded down
        f = edges.astype(np.float32)
    up = f.astype(np.float64) > edges
    f[up] = np.nextafter(f[up], np.float32(-np.inf))
    return f


def _key32(f):
    f = np.where(f == 0, np.float32(0.0), f).astype(np.float32)
    k = f.view(np.int32).astype(np.int64)
    return np.where(k < 0, k ^ 0x7fffffff, k)


def _count_below_fp64(u, edges):
    return np.searchsorted(edges, u.astype(np.float64), side="left")


def _count_below_keys(u, edges):
    return np.searchsorted(_key32(_rd(edges)), _key32(u), side="left")


def test_rounded_down_float_keys_bin_like_fp64():
    rng = np.random.default_rng(0)
    edges = np.asarray(setconf.enginit_bins(1)["uvcrd"], np.float64)
    # energies on and around every edge, plus a spread of values
    near = np.concatenate([edges, np.nextafter(edges, np.inf), np.nextafter(edges, -np.inf)]).astype(np.float32)
    near = np.concatenate([near, np.nextafter(near, np.float32(np.inf)), np.nextafter(near, np.float32(-np.inf))])
    spread = np.concatenate([rng.normal(0, 1, 20000), rng.normal(0, 0.02, 20000), rng.uniform(-25, 40, 20000),
                             10 ** rng.uniform(0, 12, 5000)]).astype(np.float32)
    u = np.concatenate([near, spread, np.float32([0.0, -0.0, np.inf, 3.4e38, -3.4e38])])
    assert np.array_equal(_count_below_fp64(u, edges), _count_below_keys(u, edges))


def test_edge_cases_of_the_rounding():
    # edges a float spacing apart, signed zeros, and edges beyond the float range
    e0 = np.float64(np.float32(0.1))
    edges = np.array([-1e40, -1.0, -0.0, 0.0, np.nextafter(e0, -1), e0, np.nextafter(e0, 1), 1e39], np.float64)
    edges = np.sort(edges)
    f = np.float32(e0)
    u = np.float32([-np.inf, -3.4e38, -1.0, -0.0, 0.0, 1e-45, np.nextafter(f, np.float32(0)), f,
                    np.nextafter(f, np.float32(1)), 3.4e38, np.inf])
    assert np.array_equal(_count_below_fp64(u, edges), _count_below_keys(u, edges))
