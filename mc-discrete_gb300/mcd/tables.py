"""Energy-loss CDF tables: host grid search, GPU FP64 fill.

The W and E grids are chosen on the host exactly as the reference chooses
them (MC/tools/probTables.py:165-411): a QUADPACK integral of dsigma/dW is
the reference value, and the number of grid points is the first of
100, 1000, ... 1e6 (then refined in tenths) whose float32 trapezoid sum is
within the tolerance.  Those checks are evaluated with the reference's
float32 arithmetic (float32 grids and integrands under NumPy's scalar
promotion rules), so the chosen sizes match the reference's.  The CDF fill
itself runs on the GPU in FP64 (mcd_build_table).

Only the two tables the DS transport samples are built: the valence
(Moller) table and the outermost shell's Gryzinski table, which the
reference uses for every Gryzinski event (MC/tools/scattering.py:625,
MC/tools/probTables.py:579).
"""
import math

import numpy as np

from . import _lib

PI_EFOUR = 6.51408491409531e-14


class TableBuildError(RuntimeError):
    """The reference's grid search has no answer (it raises there too)."""


# ---------------------------------------------------------------------------
# dsigma/dW, float64 scalars (the quad integrand, MC/tools/extFunctions.py:159-219)
# ---------------------------------------------------------------------------
def _moller64(E, W, nfree):
    eps = W / E
    if not eps < 1.0:
        return 0.0
    return nfree * PI_EFOUR * (1.0 / (eps ** 2) + (1.0 / ((1.0 - eps) ** 2)) - (1.0 / (eps * (1.0 - eps)))) / E ** 3


def _gryz64(E, W, nsi, Ebi):
    eps = W / E
    epsB = Ebi / E
    if not (eps < 1.0 and epsB < 1.0):
        return 0.0
    return (nsi * PI_EFOUR * eps * (1.0 + epsB) ** (-1.5) * (1.0 - eps) ** (epsB / (epsB + eps))
            * ((1.0 - epsB) + 4.0 * epsB * math.log(2.7 + ((1.0 - eps) / epsB) ** 0.5) / (3.0 * eps)) / (W ** 3))


# ---------------------------------------------------------------------------
# dsigma/dW in the reference's float32 arithmetic.  `E` is either a Python
# float (W-grid check) or an np.float32 (E-grid check); W is a float32 array.
# ---------------------------------------------------------------------------
F32 = np.float32


def _moller32(E, W, nfree, e_is_f32):
    E32 = F32(E)
    eps = (W / E32).astype(F32)
    one = F32(1.0)
    s = (one / np.square(eps) + one / np.square(one - eps)) - one / (eps * (one - eps))
    e3 = np.power(E32, F32(3)) if e_is_f32 else F32(float(E) ** 3)
    v = (F32(nfree * PI_EFOUR) * s) / e3
    return np.where(eps < one, v, F32(0)).astype(F32)


def _gryz32(E, W, nsi, Ebi, e_is_f32):
    E32 = F32(E)
    one = F32(1.0)
    eps = (W / E32).astype(F32)
    if e_is_f32:
        epsB = F32(Ebi) / E32
        cB = np.power(F32(one + epsB), F32(-1.5))
        k4 = F32(4.0) * epsB
        lead = one - epsB
    else:
        epsB64 = Ebi / float(E)
        epsB = F32(epsB64)
        cB = F32((1.0 + epsB64) ** (-1.5))
        k4 = F32(4.0 * epsB64)
        lead = F32(1.0 - epsB64)
    expo = epsB / (epsB + eps)
    v = F32(nsi * PI_EFOUR) * eps
    v = v * cB
    v = v * np.power(one - eps, expo)
    inner = F32(2.7) + np.sqrt((one - eps) / epsB)
    br = lead + (k4 * np.log(inner)) / (F32(3.0) * eps)
    v = v * br / np.power(W, F32(3))
    return np.where((eps < one) & (epsB < one), v, F32(0)).astype(F32)


def _trapz32(y, x):
    d = (x[1:] - x[:-1]).astype(F32)
    return F32(np.sum((d * (y[1:] + y[:-1]) / F32(2.0)).astype(F32), dtype=F32))


# ---------------------------------------------------------------------------
# grid search (MC/tools/probTables.py:54-64, 165-411)
# ---------------------------------------------------------------------------
def _orders_of_mag(max_size=1000000, num=5):
    for n in np.geomspace(100, max_size, num=num, dtype=int):
        yield int(n)


def _percents(max_size, num=10):
    for n in np.linspace(max_size / 10, max_size, num, dtype=np.float32):
        yield int(n)


class _Spec:
    def __init__(self, kind, mat, E0, Emin, Wc, tol_E, tol_W):
        self.kind = kind
        self.Ef = float(mat.fermi_e)
        self.tol_E = tol_E
        self.tol_W = tol_W
        if kind == "Moller":
            self.Wmin = float(Wc)
            self.nfree = float(mat.n_val)
            self.Eb = None
            self.Emin, self.Emax = float(Emin), float(E0)
            self.shell = mat.n_shells - 1
        else:
            k = mat.n_shells - 1
            self.shell = k
            self.Wmin = float(mat.shell_E[k])
            self.nfree = float(mat.shell_n[k])
            self.Eb = float(mat.shell_E[k])
            self.Emin = max(float(Emin), self.Wmin) if float(Emin) < self.Wmin else float(Emin)
            self.Emax = float(E0)

    def wmax(self, E):
        return (E - self.Ef) * 0.5

    def f64(self, E, W):
        if self.kind == "Moller":
            return _moller64(E, W, self.nfree)
        return _gryz64(E, W, self.nfree, self.Eb)

    def f32(self, E, W, e_is_f32):
        if self.kind == "Moller":
            return _moller32(E, W, self.nfree, e_is_f32)
        return _gryz32(E, W, self.nfree, self.Eb, e_is_f32)


def _quad(spec, E):
    from scipy.integrate import quad
    val, err = quad(lambda W: spec.f64(E, W), spec.Wmin, spec.wmax(E), limit=300, epsabs=1e-34)
    return val, err


def _first_passing(gen, make, test):
    for n in gen:
        series = make(n)
        if test(series):
            return n, series
    raise TableBuildError("no grid size up to 1e6 meets the tolerance")


def find_W_series(spec):
    """findWseries(Emax) (MC/tools/probTables.py:280-328)."""
    E = spec.Emax
    Wmax = spec.wmax(E)
    ref, err = _quad(spec, E)
    if not err < spec.tol_W * ref:
        raise TableBuildError("the W tolerance is below the quadrature error")

    def test(series):
        t = _trapz32(spec.f32(E, series, False), series)
        diff = F32(abs(F32(t - F32(ref))) / F32(ref))
        return bool(diff < F32(spec.tol_W))

    def make(n):
        return np.geomspace(spec.Wmin, Wmax, num=n, dtype=np.float32)

    n1, _ = _first_passing(_orders_of_mag(1000000), make, test)
    _, series = _first_passing(_percents(n1), make, test)
    if not np.all(series < E):
        raise TableBuildError("a W grid value is not below E0")
    return series


def find_E_series(spec, Ws):
    """findEseries(Ws[1]) (MC/tools/probTables.py:332-382)."""
    ref, _ = _quad(spec, spec.Emax)

    def test(Eseries):
        E = Eseries[-2]                          # np.float32
        wmax = F32((E - F32(spec.Ef)) * F32(0.5))
        Wsel = Ws[Ws <= wmax]
        t = _trapz32(spec.f32(E, Wsel, True), Wsel)
        diff = F32(abs(F32(t - F32(ref))) / F32(ref))
        return bool(diff < F32(spec.tol_E))

    n1, _ = _first_passing(_orders_of_mag(1000000),
                           lambda n: np.geomspace(spec.Emin, spec.Emax, num=n, dtype=np.float32), test)
    _, series = _first_passing(_percents(n1),
                               lambda n: np.linspace(spec.Emin, spec.Emax, num=n, dtype=np.float32), test)
    return series


def find_grids(kind, mat, E0, Emin, Wc, tol_E, tol_W):
    """(Ws, Es) float32 grids of one table, as the reference chooses them."""
    spec = _Spec(kind, mat, E0, Emin, Wc, tol_E, tol_W)
    Ws = find_W_series(spec)
    Es = find_E_series(spec, Ws)
    return Ws, Es


# ---------------------------------------------------------------------------
# device tables
# ---------------------------------------------------------------------------
class DeviceTable:
    """One sampled table resident on the GPU (torch tensors own the memory)."""

    def __init__(self, kind, mat, Ws, Es, device, stream=None, keep_fp64=False):
        import torch
        self.kind = kind
        self.Ws_host = np.ascontiguousarray(Ws, dtype=np.float32)
        self.Es_host = np.ascontiguousarray(Es, dtype=np.float32)
        self.nW = int(self.Ws_host.size)
        self.nE = int(self.Es_host.size)
        self.device = torch.device(device)
        self.Ws = torch.from_numpy(self.Ws_host).to(self.device)
        self.Es = torch.from_numpy(self.Es_host).to(self.device)
        self.cdf = torch.empty((self.nE, self.nW - 1), dtype=torch.float32, device=self.device)
        self.nvalid = torch.empty(self.nE, dtype=torch.int32, device=self.device)
        # uint16 column indices (held in an int16 tensor of the same bytes);
        # rows wider than 65535 columns go without a guide
        self.guide = (torch.empty((self.nE, _lib.GUIDE + 1), dtype=torch.int16, device=self.device)
                      if self.nW - 1 <= 65535 else None)
        self.cdf64 = (torch.empty((self.nE, self.nW - 1), dtype=torch.float64, device=self.device)
                      if keep_fp64 else None)
        st = stream if stream is not None else torch.cuda.current_stream(self.device)
        code = _lib.lib().mcd_build_table(
            _lib.TABLE_MOLLER if kind == "Moller" else _lib.TABLE_GRYZ,
            _lib.C.byref(mat), mat.n_shells - 1, self.nE, self.nW,
            self.Es.data_ptr(), self.Ws.data_ptr(), self.cdf.data_ptr(),
            self.cdf64.data_ptr() if self.cdf64 is not None else None,
            self.nvalid.data_ptr(), self.guide.data_ptr() if self.guide is not None else None, st.cuda_stream)
        _lib.check("mcd_build_table", code)
        self.struct = _lib.Table(self.Es.data_ptr(), self.Ws.data_ptr(), self.cdf.data_ptr(),
                                 self.nvalid.data_ptr(), self.guide.data_ptr() if self.guide is not None else None,
                                 self.nE, self.nW,
                                 float(self.Es_host[0]), float(self.Es_host[-1]))


_CACHE = {}


def ds_tables(mat, E0, Emin, Wc, tol_E, tol_W, device="cuda"):
    """(Moller, outer-shell Gryzinski) device tables, cached per parameters."""
    key = (bytes(mat.species), float(E0), float(Emin), float(Wc), float(tol_E), float(tol_W), str(device))
    t = _CACHE.get(key)
    if t is None:
        Wm, Em = find_grids("Moller", mat, E0, Emin, Wc, tol_E, tol_W)
        Wg, Eg = find_grids("Gryz", mat, E0, Emin, Wc, tol_E, tol_W)
        t = (DeviceTable("Moller", mat, Wm, Em, device), DeviceTable("Gryz", mat, Wg, Eg, device))
        _CACHE[key] = t
    return t


_SIG_CACHE = {}


SIG64_CELLS = 256


def sig64_stride(n_channels):
    """Doubles per cell record of an FP64 table: a flag word, a pad word and
    four cubic coefficients per column."""
    return 2 + 4 * n_channels


def sigma_table_fits(sim, mat):
    """Does the FP64 table of this simulation's energy range fit the buffer
    (mcd_sigma_table_bytes)?  One block of 256 cell records per octave of
    (Emin, E0], each of 2 + 4 (n_shells + 3) doubles."""
    octaves = math.frexp(float(sim.E0))[1] - math.frexp(float(sim.Emin))[1] + 1
    return 8 * octaves * SIG64_CELLS * sig64_stride(mat.n_shells + 3) <= _lib.lib().mcd_sigma_table_bytes()


def sigma_table(sim, mat, device="cuda"):
    """Device cross-section table of a DS simulation for its precision
    (mcd_build_sigma_table over [Emin, E0]: FP32, E times the total and the
    running channel cross sections on a log2-E grid; FP64, the mean free
    path and the running sums as fractions of the total, cubics on octave
    grids),
    cached per material, Wc, elastic model, density scale, energy range and
    precision."""
    import torch
    key = (bytes(mat), int(sim.elastic), float(sim.Wc), float(sim.n_scale), float(sim.E0), float(sim.Emin),
           int(sim.precision), str(device))
    t = _SIG_CACHE.get(key)
    if t is None:
        t = torch.empty(_lib.lib().mcd_sigma_table_bytes() // 4, dtype=torch.float32, device=device)
        st = torch.cuda.current_stream(t.device)
        code = _lib.lib().mcd_build_sigma_table(_lib.C.byref(sim), _lib.C.byref(mat), t.data_ptr(), st.cuda_stream)
        _lib.check("mcd_build_sigma_table", code)
        _SIG_CACHE[key] = t
    return t
