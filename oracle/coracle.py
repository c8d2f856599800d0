"""ctypes driver of the C oracle (oracle/_build/libmcd_oracle.so).

TEST INFRASTRUCTURE ONLY (tests, __graft_entry__.smoke, bench.py's CPU leg).
Material constants and tables come from oracle/mcd_oracle.py, so the C
oracle shares nothing with the library under test.
"""
import ctypes as C
import os
import subprocess

import numpy as np

import mcd_oracle as O

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libmcd_oracle.so")
MAX_SHELLS = 8


class Mat(C.Structure):
    _fields_ = [("Z", C.c_double), ("n_val", C.c_double), ("E_val", C.c_double), ("atnd", C.c_double),
                ("plasmon_e", C.c_double), ("fermi_e", C.c_double), ("J", C.c_double), ("bethe_k", C.c_double),
                ("n_shells", C.c_int), ("shell_E", C.c_double * MAX_SHELLS),
                ("shell_n", C.c_double * MAX_SHELLS), ("xip_g", C.c_double)]


class Tab(C.Structure):
    _fields_ = [("Es", C.c_void_p), ("Ws", C.c_void_p), ("cdf", C.c_void_p), ("nE", C.c_int), ("nW", C.c_int)]


class Sim(C.Structure):
    _fields_ = [("mode", C.c_int), ("bethe", C.c_int), ("E0", C.c_double), ("Emin", C.c_double),
                ("tilt", C.c_double), ("Wc", C.c_double), ("thickness", C.c_double),
                ("max_scatt", C.c_longlong), ("seed", C.c_ulonglong), ("sim_id", C.c_uint),
                ("quirks", C.c_uint), ("J_scale", C.c_double), ("n_scale", C.c_double),
                ("elastic", C.c_int), ("diff", C.c_int)]


class Out(C.Structure):
    _fields_ = [("outcome", C.c_void_p), ("flags", C.c_void_p), ("final_E", C.c_void_p), ("dir", C.c_void_p),
                ("last_pos", C.c_void_p), ("max_z", C.c_void_p), ("n_events", C.c_void_p),
                ("channel", C.c_void_p), ("nan_events", C.c_void_p)]


_LIB = None


def build():
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _LIB
    if _LIB is None:
        src = os.path.join(HERE, "mcd_oracle.c")
        if not os.path.exists(LIB_PATH) or os.path.getmtime(LIB_PATH) < os.path.getmtime(src):
            build()
        _LIB = C.CDLL(LIB_PATH)
        _LIB.mco_run.restype = C.c_int
        _LIB.mco_run.argtypes = [C.POINTER(Sim), C.POINTER(Mat), C.POINTER(Tab), C.POINTER(Tab),
                                 C.c_ulonglong, C.c_longlong, C.POINTER(Out), C.c_int]
    return _LIB


def mat_struct(mat):
    m = Mat()
    m.Z = mat.Z
    m.n_val = mat.n_val
    m.E_val = mat.E_val
    m.atnd = mat.atnd
    m.plasmon_e = mat.plasmon_e
    m.fermi_e = mat.fermi_e
    m.J = mat.J
    m.bethe_k = mat.bethe_k
    m.n_shells = len(mat.shells)
    for k, (_, Es, ns) in enumerate(mat.shells):
        m.shell_E[k] = Es
        m.shell_n[k] = ns
    m.xip_g = mat.xip_g or 0.0
    return m


class HostTable:
    """float32 grids + float32 CDF (0 = masked) kept alive for the C call."""

    def __init__(self, Ws, Es, cdf32):
        self.Ws = np.ascontiguousarray(Ws, dtype=np.float32)
        self.Es = np.ascontiguousarray(Es, dtype=np.float32)
        self.cdf = np.ascontiguousarray(cdf32, dtype=np.float32)
        self.struct = Tab(self.Es.ctypes.data, self.Ws.ctypes.data, self.cdf.ctypes.data, self.Es.size,
                          self.Ws.size)

    @classmethod
    def build(cls, kind, mat, Ws, Es):
        cdf, valid = O.table_cdf(kind, mat, Ws, Es)
        return cls(Ws, Es, O.table_store32(cdf, valid))


BETHE = {"classical": 0, "JL": 1, "explicit": 2}
ELASTIC = list(O.ELASTIC_MODELS)


def run(mat, E0, Emin, tilt, n, seed=0, first=0, mode="DS", Wc=100.0, tables=None, bethe="classical",
        thickness=1e30, max_scatt=10 ** 15, sim_id=0, quirks=7, J_scale=1.0, n_scale=1.0, nthreads=None,
        elastic="Ruth_vanilla", diff=False):
    """Run n electrons; returns a dict of per-electron arrays + channel counts.
    elastic is a resolved model name (mcd_oracle.ELASTIC_MODELS)."""
    L = lib()
    s = Sim(0 if mode == "DS" else 1, BETHE[bethe], E0, Emin, tilt, Wc, thickness, max_scatt, seed, sim_id,
            quirks, J_scale, n_scale, ELASTIC.index(elastic), 1 if diff else 0)
    m = mat_struct(mat)
    res = dict(outcome=np.zeros(n, np.uint8), flags=np.zeros(n, np.uint8), final_E=np.zeros(n),
               dir=np.zeros((n, 3)), last_pos=np.zeros((n, 3)), max_z=np.zeros(n),
               n_events=np.zeros(n, np.int32), channel=np.zeros(16, np.uint64), nan_events=np.zeros(1, np.uint64))
    o = Out(*[res[k].ctypes.data for k in ("outcome", "flags", "final_E", "dir", "last_pos", "max_z",
                                              "n_events", "channel", "nan_events")])
    tm = tables[0].struct if tables else None
    tg = tables[1].struct if tables else None
    rc = L.mco_run(C.byref(s), C.byref(m), C.byref(tm) if tm else None, C.byref(tg) if tg else None,
                   first, n, C.byref(o), nthreads or os.cpu_count() or 1)
    if rc != 0:
        raise RuntimeError("mco_run failed: %d" % rc)
    return res
