"""The C-ABI library: builds, loads, exports every symbol include/ermod_gpu.h declares,
and its host-only entry points behave like the reference (no GPU needed)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    text = open(os.path.join(ROOT, "include", "ermod_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(ermod_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(gpu_lib):
    from ermod_gb300 import _lib
    names = declared_functions()
    assert len(names) >= 20
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (ermod_\w+)", out))
    missing = [n for n in names if n not in exported]
    assert not missing, missing
    assert sorted(_lib.EXPORTS) == names


def test_default_params_and_status_strings(gpu_lib):
    from ermod_gb300 import _lib
    p = _lib.Params()
    gpu_lib.ermod_default_params(C.byref(p))
    assert p.abi_version == _lib.ABI_VERSION and p.cltype == 2 and p.splodr == 4
    assert p.elecut == 12.0 and p.lwljcut == 10.0 and p.upljcut == 12.0
    assert abs(p.temp - 300.0 * 8.314510e-3 / 4.184) < 1e-15
    assert b"eng_min" in gpu_lib.ermod_status_string(_lib.E_ENG_MIN)


def test_create_rejects_bad_parameters_before_touching_a_device(gpu_lib):
    from ermod_gb300 import _lib
    p = _lib.Params()
    gpu_lib.ermod_default_params(C.byref(p))
    ctx = C.c_void_p()
    bad = _lib.Params.from_buffer_copy(p)
    bad.cltype = 1  # Ewald: the reference itself stops on it (setconf.F90:329-331)
    assert gpu_lib.ermod_create(C.byref(bad), 0, C.byref(ctx)) == _lib.E_UNSUPPORTED
    bad = _lib.Params.from_buffer_copy(p)
    bad.abi_version = 99
    assert gpu_lib.ermod_create(C.byref(bad), 0, C.byref(ctx)) == _lib.E_PARAM
    bad = _lib.Params.from_buffer_copy(p)
    bad.screen = 0.34
    bad.lwljcut = 13.0
    assert gpu_lib.ermod_create(C.byref(bad), 0, C.byref(ctx)) == _lib.E_PARAM


def test_engstore_merge_matches_reference_formulas(gpu_lib):
    """engstore (engproc.F90:475-560): voffset max + rescale, sums, min/max, /engnorm."""
    from ermod_gb300 import _lib
    rng = np.random.default_rng(3)
    nrank, E, S, N = 3, 7, 4, 2
    temp = 0.596
    edens = rng.random((nrank, E))
    ecorr = rng.random((nrank, E * E))
    eself = rng.random((nrank, S))
    slnuv = rng.random((nrank, N))
    mn = rng.random((nrank, N + 1))
    mx = mn + 1
    sc = np.zeros((nrank, 5))
    sc[:, 0] = rng.random(nrank) + 1
    sc[:, 1] = [10, 20, 30]
    sc[:, 2] = rng.random(nrank) + 1
    sc[:, 3] = [-1.0, -0.5, -0.8]
    sc[:, 4] = 1
    for slttype in (1, 2):
        ed, ec, es, sl, a, b, s = (x.copy() for x in (edens, ecorr, eself, slnuv, mn, mx, sc))
        st = gpu_lib.ermod_engstore_merge(nrank, slttype, 1, temp, E, S, N, _lib.dp(ed), _lib.dp(ec), _lib.dp(es),
                                          _lib.dp(sl), _lib.dp(a), _lib.dp(b), _lib.dp(s))
        assert st == 0
        vmax = sc[:, 3].max()
        scale = np.exp((sc[:, 3] - vmax) / temp) if slttype == 1 else np.exp(-(sc[:, 3] - vmax) / temp)
        engnorm = (sc[:, 0] * scale).sum()
        np.testing.assert_allclose(s[0, 0], engnorm, rtol=1e-14)
        np.testing.assert_allclose(ed[0], (edens * scale[:, None]).sum(0) / engnorm, rtol=1e-13)
        np.testing.assert_allclose(ec[0], (ecorr * scale[:, None]).sum(0) / engnorm, rtol=1e-13)
        np.testing.assert_allclose(es[0], (eself * scale[:, None]).sum(0) / engnorm, rtol=1e-13)
        np.testing.assert_allclose(a[0], mn.min(0))
        np.testing.assert_allclose(b[0], mx.max(0))
        assert s[0, 1] == 60 and s[0, 3] == vmax
        np.testing.assert_allclose(s[0, 2], sc[:, 2].sum() / engnorm, rtol=1e-14)
