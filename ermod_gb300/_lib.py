"""ctypes binding of ``libermod_gb300.so`` (the C ABI declared in ``include/ermod_gpu.h``).

The library is built in-tree by ``ermod_gb300.build``.  Loading never falls back to
anything: a missing or stale library raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libermod_gb300.so")

OK = 0
E_ENG_MIN, E_ENG_SFT, E_ENG_BUG, E_ENG_CNS, E_RCP_CNS, E_RCP_FST = 101, 102, 103, 104, 105, 106
E_INS_GEO, E_SET_PRS, E_ENG_SLB = 107, 108, 109
W_MBIN, E_INS_SIZ = 110, 111
E_PARAM, E_NONCUBOID, E_UNSUPPORTED = 120, 121, 122
E_CUDA, E_CUFFT, E_NOMEM, E_DEVICE = 130, 131, 132, 133
PRECISION_FP64, PRECISION_MIXED = 0, 1
ABI_VERSION = 2

# halt_with_error identities (mpiproc.F90:203-264) of the status codes
REFERENCE_CODE = {E_ENG_MIN: "eng_min", E_ENG_SFT: "eng_sft", E_ENG_BUG: "eng_bug", E_ENG_CNS: "eng_cns",
                  E_RCP_CNS: "rcp_cns", E_RCP_FST: "rcp_fst", E_INS_GEO: "ins_geo", E_SET_PRS: "set_prs",
                  E_ENG_SLB: "eng_slb", W_MBIN: "mbin", E_INS_SIZ: "ins_siz"}


class Params(C.Structure):
    _fields_ = [
        ("abi_version", C.c_int32), ("slttype", C.c_int32), ("estype", C.c_int32), ("cltype", C.c_int32),
        ("ljswitch", C.c_int32), ("splodr", C.c_int32), ("ms1max", C.c_int32), ("ms2max", C.c_int32),
        ("ms3max", C.c_int32), ("wgtslf", C.c_int32), ("corrcal", C.c_int32), ("selfcal", C.c_int32),
        ("force_calculation", C.c_int32), ("precision", C.c_int32), ("batch", C.c_int32),
        ("count_mirror", C.c_int32),
        ("elecut", C.c_double), ("lwljcut", C.c_double), ("upljcut", C.c_double), ("screen", C.c_double),
        ("temp", C.c_double), ("block_threshold", C.c_double), ("boxshp", C.c_int32), ("finish_group", C.c_int32),
    ]


class InsertParams(C.Structure):
    _fields_ = [("insposition", C.c_int32), ("insorient", C.c_int32), ("insorigin", C.c_int32),
                ("pad_", C.c_int32), ("lwreg", C.c_double), ("upreg", C.c_double), ("seed", C.c_uint64),
                ("offset", C.c_uint64)]


EXPORTS = [
    "ermod_default_params", "ermod_create", "ermod_destroy", "ermod_set_stream", "ermod_set_topology",
    "ermod_set_bins", "ermod_frame", "ermod_frame_device", "ermod_placements", "ermod_placements_device",
    "ermod_sync", "ermod_clear", "ermod_get_accum", "ermod_get_sizes", "ermod_error_info",
    "ermod_timing_enable", "ermod_timing_reset", "ermod_timing_get", "ermod_last_error_string",
    "ermod_status_string", "ermod_enginit_species", "ermod_getscrn", "ermod_lj_tables", "ermod_engstore_merge",
    "ermod_ecorr_add_noalloc", "ermod_adjoint_enable", "ermod_adjoint_get", "ermod_graph_create",
    "ermod_graph_launch", "ermod_graph_sync", "ermod_graph_destroy", "ermod_write_engdist",
    "ermod_write_selfdist", "ermod_write_corr", "ermod_write_uvrange", "ermod_format_g",
    "ermod_generate_placements", "ermod_intermediate_enable", "ermod_intermediate_get",
    "ermod_set_configuration_check", "ermod_set_aggregate", "ermod_set_reference_structure",
    "ermod_set_solute_library",
]

_lib = None


def load(path: str = LIB_PATH):
    """Load the library (raises OSError when it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise OSError(f"{path} is missing: run `python -m ermod_gb300.build` (nvcc, sm_103a)")
    L = C.CDLL(path)
    dp, ip, vp = C.POINTER(C.c_double), C.POINTER(C.c_int), C.c_void_p
    i64p = C.POINTER(C.c_int64)
    L.ermod_default_params.argtypes = [C.POINTER(Params)]
    L.ermod_default_params.restype = None
    L.ermod_create.argtypes = [C.POINTER(Params), C.c_int, C.POINTER(vp)]
    L.ermod_destroy.argtypes = [vp]
    L.ermod_set_stream.argtypes = [vp, vp]
    L.ermod_set_topology.argtypes = [vp, C.c_int, C.c_int, ip, ip, ip, dp, ip, C.c_int, dp, dp]
    L.ermod_set_bins.argtypes = [vp, C.c_int, ip, ip, dp, C.c_int, dp]
    L.ermod_frame.argtypes = [vp, dp, dp, C.c_double]
    L.ermod_frame_device.argtypes = [vp, vp, dp, C.c_double]
    L.ermod_placements.argtypes = [vp, C.c_int, ip, dp, dp, dp, dp]
    L.ermod_placements_device.argtypes = [vp, C.c_int, vp, vp, vp, vp, vp]
    L.ermod_sync.argtypes = [vp]
    L.ermod_clear.argtypes = [vp]
    L.ermod_get_accum.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, i64p]
    L.ermod_get_sizes.argtypes = [vp, ip, ip, ip, ip]
    L.ermod_error_info.argtypes = [vp, ip, ip, dp]
    L.ermod_timing_enable.argtypes = [vp, C.c_int]
    L.ermod_timing_reset.argtypes = [vp]
    L.ermod_timing_get.argtypes = [vp, C.c_int, dp, C.POINTER(C.c_char_p), ip, i64p]
    L.ermod_last_error_string.restype = C.c_char_p
    L.ermod_last_error_string.argtypes = []
    L.ermod_status_string.restype = C.c_char_p
    L.ermod_status_string.argtypes = [C.c_int]
    L.ermod_enginit_species.argtypes = [dp, C.c_int, C.c_int, dp, ip, ip]
    L.ermod_getscrn.restype = C.c_double
    L.ermod_getscrn.argtypes = [C.c_double, C.c_double, C.c_int]
    L.ermod_lj_tables.argtypes = [C.c_int, dp, dp, C.c_int, C.c_int, C.c_int, ip, ip, dp, dp]
    L.ermod_engstore_merge.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, C.c_int, C.c_int, dp, dp,
                                       dp, dp, dp, dp, dp]
    L.ermod_ecorr_add_noalloc.argtypes = [vp, vp, C.c_int, C.c_int, vp, vp, vp]
    L.ermod_adjoint_enable.argtypes = [vp, C.c_int, C.c_int]
    L.ermod_adjoint_get.argtypes = [vp, dp, dp, ip]
    vpp = C.POINTER(vp)
    L.ermod_graph_create.argtypes = [C.c_int, vpp, vpp, dp, dp, ip, ip, vpp, vpp, vpp, C.POINTER(vp)]
    L.ermod_graph_launch.argtypes = [vp, vp]
    L.ermod_graph_sync.argtypes = [vp]
    L.ermod_graph_destroy.argtypes = [vp]
    L.ermod_write_engdist.argtypes = [C.c_char_p, C.c_int, ip, ip, dp, dp]
    L.ermod_write_selfdist.argtypes = [C.c_char_p, C.c_int, dp, dp]
    L.ermod_write_corr.argtypes = [C.c_char_p, C.c_int, dp]
    L.ermod_write_uvrange.argtypes = [C.c_char_p, C.c_int, dp, dp]
    L.ermod_format_g.argtypes = [C.c_double, C.c_int, C.c_int, C.c_char_p, C.c_int]
    L.ermod_generate_placements.argtypes = [vp, C.c_int, C.c_int, dp, dp, C.POINTER(InsertParams), vp, vp]
    L.ermod_intermediate_enable.argtypes = [vp, dp]
    L.ermod_intermediate_get.argtypes = [vp, dp, dp, dp]
    L.ermod_set_configuration_check.argtypes = [vp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_double, C.c_double]
    L.ermod_set_aggregate.argtypes = [vp, ip, dp]
    L.ermod_set_reference_structure.argtypes = [vp, ip, dp, dp, C.c_int, dp, dp]
    L.ermod_set_solute_library.argtypes = [vp, C.c_int, C.c_int, dp, C.c_int, dp, C.c_int, C.c_double, C.c_double]
    _lib = L
    return L


def dp(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_double))


def ip(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int))


def i64p(a):
    return None if a is None else a.ctypes.data_as(C.POINTER(C.c_int64))


class ErmodError(RuntimeError):
    """A nonzero ermod_status; ``.code`` is the status, ``.name`` the reference identity."""

    def __init__(self, code: int, where: str):
        L = load()
        msg = L.ermod_status_string(code).decode()
        detail = L.ermod_last_error_string().decode()
        super().__init__(f"{where}: {msg} (status {code}){' -- ' + detail if detail else ''}")
        self.code = code
        self.name = REFERENCE_CODE.get(code, "")


def check(code: int, where: str):
    if code != OK:
        raise ErmodError(code, where)
