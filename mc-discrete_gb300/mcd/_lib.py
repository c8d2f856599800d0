"""ctypes binding of libmcd.so (the C ABI declared in include/mcd.h).

The library is loaded from mcd/_lib/libmcd.so, built in-tree by mcd.build.
There is no CPU fallback: every device entry point raises if the library
cannot be loaded or a call fails.
"""
import ctypes as C
import os

from . import build as _build

ABI_VERSION = 10
MAX_SHELLS = 8
GUIDE = 256
MAX_CHANNELS = 16
HIST_E_MAX = 256
HIST_T_MAX = 180

OK, EINVAL, ECUDA, ETOOBIG, ENOSPECIES, ENODEV = range(6)

FLAG_TABLE_RANGE = 0x01
FLAG_RING_FULL = 0x02
FLAG_NAN = 0x04
FLAG_CLAMPED = 0x08
FLAG_LONG_PATH = 0x10
FLAG_LONG = 0x20
FLAG_RING_INDEX = 0x40

OUT_NONE, OUT_BKS, OUT_ABS, OUT_TRSM, OUT_TRDF, OUT_LONG = range(6)
OUTCOME_NAMES = ("none", "bks", "abs", "trsm", "trdf", "long")
CH_RUTH, CH_MOLLER, CH_QUINN, CH_GRYZ0, CH_DIFF = 0, 1, 2, 3, 11
ELASTIC_RUTH, ELASTIC_RUTH_WDEFL, ELASTIC_NIGRAM, ELASTIC_NIGRAM_WDEFL = 0, 1, 2, 3
ELASTIC = {"Ruth_vanilla": ELASTIC_RUTH, "Ruth_vanilla_wDefl": ELASTIC_RUTH_WDEFL,
           "Ruth_nigram": ELASTIC_NIGRAM, "Ruth_nigram_wDefl": ELASTIC_NIGRAM_WDEFL}
MODE_DS, MODE_CONT = 0, 1
BETHE = {"classical": 0, "JL": 1, "explicit": 2}
FP32, FP64 = 0, 1
ADJ_EXIT_E, ADJ_MAX_DEPTH = 0, 1
# event-ring record fields (after the electron / event-and-channel header)
EV_E, EV_W, EV_PATHL, EV_C2, EV_PHI, EV_POS = 0x01, 0x02, 0x04, 0x08, 0x10, 0x20
EV_ALL = 0x3f
EV_PACKED_HEAD = 0x40   # one-word record header: electron << 4 | channel
TABLE_MOLLER, TABLE_GRYZ = 0, 1

Q_CROSSING_STEP = 0x1
Q_HALF_PHI_FOLD = 0x2
Q_NAN_DIRECTION = 0x4
QUIRKS_REFERENCE = 0x7
TALLY_CHANNELS = 0x1


class Material(C.Structure):
    _fields_ = [
        ("species", C.c_char * 8),
        ("name_val", C.c_char * 16),
        ("shell_name", (C.c_char * 8) * MAX_SHELLS),
        ("Z", C.c_int32),
        ("n_shells", C.c_int32),
        ("n_val", C.c_double),
        ("E_val", C.c_double),
        ("density", C.c_double),
        ("atwt", C.c_double),
        ("bethe_k", C.c_double),
        ("atnd", C.c_double),
        ("plasmon_e", C.c_double),
        ("fermi_e", C.c_double),
        ("J", C.c_double),
        ("shell_E", C.c_double * MAX_SHELLS),
        ("shell_n", C.c_double * MAX_SHELLS),
        ("xip_g", C.c_double),
    ]


class Table(C.Structure):
    _fields_ = [
        ("Es", C.c_void_p),
        ("Ws", C.c_void_p),
        ("cdf", C.c_void_p),
        ("nvalid", C.c_void_p),
        ("guide", C.c_void_p),
        ("nE", C.c_int32),
        ("nW", C.c_int32),
        ("E_first", C.c_float),
        ("E_last", C.c_float),
    ]


class Sim(C.Structure):
    _fields_ = [
        ("mode", C.c_int32),
        ("bethe_model", C.c_int32),
        ("precision", C.c_int32),
        ("quirks", C.c_uint32),
        ("tally_flags", C.c_uint32),
        ("sim_id", C.c_uint32),
        ("E0", C.c_double),
        ("Emin", C.c_double),
        ("s_tilt", C.c_double),
        ("Wc", C.c_double),
        ("thickness", C.c_double),
        ("max_scatt", C.c_int64),
        ("num_el", C.c_int64),
        ("first_electron", C.c_uint64),
        ("seed", C.c_uint64),
        ("hist_E_bins", C.c_int32),
        ("hist_T_bins", C.c_int32),
        ("hist_E_width", C.c_double),
        ("hist_T_width", C.c_double),
        ("J_scale", C.c_double),
        ("n_scale", C.c_double),
        ("elastic", C.c_int32),
        ("diff_mfp", C.c_int32),
        ("sigma_table", C.c_void_p),
        ("electrons", C.c_void_p),   # host address of an ElectronOut (batched runs)
    ]


class Tally(C.Structure):
    _fields_ = [
        ("outcome", C.c_uint64 * 8),
        ("events", C.c_uint64),
        ("double_rows", C.c_uint64),
        ("nan_events", C.c_uint64),
        ("clamped", C.c_uint64),
        ("long_path", C.c_uint64),
        ("table_range", C.c_uint64),
        ("channel", C.c_uint64 * MAX_CHANNELS),
        ("sum_E_bks", C.c_double),
        ("sum_E2_bks", C.c_double),
        ("sum_steps2", C.c_double),
        ("reserved", C.c_double),
        ("hist_E", C.c_uint64 * HIST_E_MAX),
        ("hist_T", C.c_uint64 * HIST_T_MAX),
    ]


class ElectronOut(C.Structure):
    _fields_ = [
        ("outcome", C.c_void_p),
        ("flags", C.c_void_p),
        ("final_E", C.c_void_p),
        ("dir", C.c_void_p),
        ("last_pos", C.c_void_p),
        ("max_z", C.c_void_p),
        ("n_events", C.c_void_p),
    ]


class Event(C.Structure):
    _fields_ = [
        ("electron", C.c_uint32),
        ("step_chan", C.c_uint32),
        ("E", C.c_float),
        ("W", C.c_float),
        ("pathl", C.c_float),
        ("c2", C.c_float),
        ("half_phi", C.c_float),
        ("x", C.c_float),
        ("y", C.c_float),
        ("z", C.c_float),
    ]


class EventRing(C.Structure):
    _fields_ = [
        ("rec", C.c_void_p),
        ("capacity", C.c_uint64),
        ("cursor", C.c_void_p),
        ("fields", C.c_uint32),
        ("reserved", C.c_uint32),
    ]


class Tune(C.Structure):
    _fields_ = [
        ("block_size", C.c_int32),
        ("blocks_per_sm", C.c_int32),
        ("refill", C.c_int32),
        ("variant", C.c_int32),
        ("reserved", C.c_int64),
    ]


class SoftHist(C.Structure):
    _fields_ = [("nbins", C.c_int32), ("quantity", C.c_int32), ("lo", C.c_double), ("hi", C.c_double),
                ("sigma", C.c_double)]


class AdjointBuf(C.Structure):
    _fields_ = [("ckpt", C.c_void_p), ("kstar", C.c_void_p), ("E_exit", C.c_void_p), ("max_ckpt", C.c_int32),
                ("reserved", C.c_int32), ("queue", C.c_void_p)]


STRUCTS = {
    "mcd_material": Material,
    "mcd_table": Table,
    "mcd_sim": Sim,
    "mcd_tally": Tally,
    "mcd_electron_out": ElectronOut,
    "mcd_event": Event,
    "mcd_event_ring": EventRing,
    "mcd_tune": Tune,
    "mcd_softhist": SoftHist,
    "mcd_adjoint_buf": AdjointBuf,
}

# name -> (restype, argtypes)
SIGNATURES = {
    "mcd_abi_version": (C.c_int, []),
    "mcd_strerror": (C.c_char_p, [C.c_int]),
    "mcd_struct_size": (C.c_size_t, [C.c_char_p]),
    "mcd_material_init": (C.c_int, [C.c_char_p, C.POINTER(Material)]),
    "mcd_device_info": (C.c_int, [C.POINTER(C.c_int)] * 3),
    "mcd_build_table": (C.c_int, [C.c_int, C.POINTER(Material), C.c_int, C.c_int32, C.c_int32,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_void_p]),
    "mcd_run": (C.c_int, [C.POINTER(Sim), C.POINTER(Material), C.POINTER(Table), C.POINTER(Table),
                          C.c_void_p, C.POINTER(ElectronOut), C.POINTER(EventRing), C.c_void_p,
                          C.c_int32, C.c_void_p]),
    "mcd_sigma_table_bytes": (C.c_size_t, []),
    "mcd_build_sigma_table": (C.c_int, [C.POINTER(Sim), C.POINTER(Material), C.c_void_p, C.c_void_p]),
    "mcd_batch_workspace_bytes": (C.c_size_t, [C.c_int32]),
    "mcd_batch_upload_bytes": (C.c_size_t, [C.c_int32]),
    "mcd_batch_prepare": (C.c_int, [C.POINTER(Sim), C.c_int32, C.POINTER(Material), C.POINTER(C.c_int32),
                                    C.POINTER(Table), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                    C.c_void_p, C.c_size_t, C.c_void_p]),
    "mcd_run_batched": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(Tune), C.c_void_p,
                                  C.c_void_p]),
    "mcd_run_batched_noalloc": (C.c_int, [C.POINTER(Sim), C.c_int32, C.POINTER(Material), C.POINTER(C.c_int32),
                                          C.POINTER(Table), C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                          C.c_void_p, C.POINTER(Tune), C.c_void_p, C.c_void_p]),
    "mcd_event_bytes": (C.c_size_t, [C.c_uint32]),
    "mcd_project_detector": (C.c_int, [C.c_void_p, C.c_int64, C.c_int32, C.c_double, C.c_double, C.c_double,
                                       C.c_double, C.c_void_p, C.c_void_p]),
    "mcd_run_batched_ring": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(Tune), C.POINTER(EventRing),
                                       C.c_void_p, C.c_void_p]),
    "mcd_adjoint_forward": (C.c_int, [C.POINTER(Sim), C.POINTER(Material), C.POINTER(SoftHist),
                                      C.POINTER(AdjointBuf), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]),
    "mcd_adjoint": (C.c_int, [C.POINTER(Sim), C.POINTER(Material), C.POINTER(SoftHist), C.POINTER(AdjointBuf),
                              C.c_void_p, C.c_void_p, C.c_void_p]),
    "mcd_adjoint_chain": (C.c_int, [C.POINTER(Sim), C.POINTER(Material), C.POINTER(SoftHist),
                                    C.POINTER(AdjointBuf), C.c_void_p, C.c_void_p]),
}
STATIC_MAX_SIMS = 64
FLAG_CKPT = 0x80

_LIB = None


class MCDError(RuntimeError):
    def __init__(self, fn, code):
        msg = _LIB.mcd_strerror(code).decode() if _LIB is not None else str(code)
        super().__init__("%s failed: %s (code %d)" % (fn, msg, code))
        self.code = code


def lib(build_if_missing=True):
    """Load (building first if needed) and return the ctypes library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if build_if_missing and (not os.path.exists(path) or _build._stale()):
        _build.build()
    if not os.path.exists(path):
        raise RuntimeError("libmcd.so is missing at %s; run mcd.build.build()" % path)
    h = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(h, name)
        f.restype = res
        f.argtypes = args
    if h.mcd_abi_version() != ABI_VERSION:
        raise RuntimeError("libmcd ABI version mismatch")
    for name, cls in STRUCTS.items():
        n = h.mcd_struct_size(name.encode())
        if n != C.sizeof(cls):
            raise RuntimeError("layout mismatch for %s: C %d vs ctypes %d" % (name, n, C.sizeof(cls)))
    _LIB = h
    return h


def check(fn, code):
    if code != OK:
        raise MCDError(fn, code)


def material(species):
    m = Material()
    check("mcd_material_init", lib().mcd_material_init(species.encode(), C.byref(m)))
    return m
