"""engstore's output files (CPU): Fortran G fields, the engsln/engref bin layout read
back the way slvfe reads it (list-directed), and the corref unformatted record."""
import struct

import numpy as np

from ermod_gb300 import engstore, setconf


def test_fortran_g_fields():
    f = engstore.format_g
    assert f(1.5, 15, 7) == "   1.500000    "
    assert f(-20.02, 15, 7) == "  -20.02000    "
    assert f(0.0125, 15, 7) == "  0.1250000E-01"
    assert f(1.0e11, 15, 7) == "  0.1000000E+12"
    assert f(0.0, 15, 7) == "   0.000000    "
    assert f(1.0e-300, 15, 7) == "  0.1000000-299"
    assert f(123456.7, 15, 7) == "   123456.7    "
    assert f(9999999.6, 15, 7) == "  0.1000000E+08"  # rounds to 8 digits before the point
    assert f(0.099999996, 15, 7) == "  0.1000000    "  # rounds up into the F range
    assert f(2.0 / 3.0, 25, 15) == "    0.666666666666667    "
    assert len(f(-1.0 / 3.0, 25, 15)) == 25


def test_engdist_corr_and_uvrange_files(tmp_path):
    bins = setconf.enginit_bins(2)
    E = len(bins["uvcrd"])
    rng = np.random.default_rng(4)
    merged = dict(edens=rng.random(E), ecorr=rng.random((E, E)), eself=rng.random(bins["esmax"]),
                  minuv=np.array([-30.0, -12.5, -3.25]), maxuv=np.array([4.0e10, 15.0, 9.5]))
    paths = engstore.write_outputs(str(tmp_path), merged, bins, slttype=2, corrcal=1, selfcal=1)
    names = sorted(p.split("/")[-1] for p in paths)
    assert names == ["corref.tt", "engref.tt", "slfeng.tt", "uvrange.tt"]
    rows = [ln.split() for ln in open(tmp_path / "engref.tt").read().splitlines()]
    assert len(rows) == E
    crd = np.array([float(r[0]) for r in rows])
    pti = np.array([int(r[1]) for r in rows])
    dens = np.array([float(r[2]) for r in rows])
    np.testing.assert_allclose(dens, merged["edens"], rtol=1e-14)
    assert list(np.unique(pti)) == [1, 2] and np.all(np.diff(pti) >= 0)
    # repval: linear midpoint in the soft region, geometric mean beyond, last edge at the end
    u = bins["uvcrd"]
    n1, soft = bins["uvmax"][0], bins["uvsoft"][0]
    np.testing.assert_allclose(crd[0], (u[0] + u[1]) / 2, rtol=1e-6)
    np.testing.assert_allclose(crd[soft], np.sqrt(u[soft] * u[soft + 1]), rtol=1e-6)
    np.testing.assert_allclose(crd[n1 - 1], u[n1 - 1], rtol=1e-6)
    raw = open(tmp_path / "corref.tt", "rb").read()
    (head,) = struct.unpack("<I", raw[:4])
    (tail,) = struct.unpack("<I", raw[-4:])
    assert head == tail == 8 * E * E and len(raw) == 8 * E * E + 8
    back = np.frombuffer(raw[4:-4], "<f8").reshape(E, E, order="F")
    np.testing.assert_array_equal(back, merged["ecorr"])
    lines = open(tmp_path / "uvrange.tt").read().splitlines()
    assert lines[0] == " species     minimum        maximum"
    assert lines[2] == "    1      -12.50000       15.00000"
    assert lines[1].startswith("    0      -30.00000") and "E+11" in lines[1]
    self_rows = [ln.split() for ln in open(tmp_path / "slfeng.tt").read().splitlines()]
    assert len(self_rows) == bins["esmax"]
    np.testing.assert_allclose([float(r[1]) for r in self_rows], merged["eself"], rtol=1e-14)
