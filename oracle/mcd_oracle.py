"""CPU oracle for the electron-trajectory Monte Carlo (FP64 restatement).

TEST INFRASTRUCTURE ONLY.  This module is the parity reference: tests/, the smoke check
in __graft_entry__ and the CPU-baseline leg of bench.py may import it; the
library under mc-discrete_gb300/ never does.

It restates, function by function, the arithmetic of the reference
elena-pascal/MC-discrete (paths below are relative to that project):

  material constants       MC/tools/material.py:15-90,117-133,151-302
  total cross sections     MC/tools/crossSections.py:14-27,37-58,183-284
  stopping powers          MC/tools/stoppingPowers.py:112-215
  dsigma/dW                MC/tools/extFunctions.py:159-219
  CDF table fill           MC/tools/probTables.py:415-462 (+ maxW :17-41)
  table sampling           MC/tools/scattering.py:63-94
  angles                   MC/tools/scattering.py:125-179
  DS event + trajectory    MC/tools/scattering.py:440-679,
                           MC/tools/singleScatter.py:10-41
  continuous trajectory    MC/tools/scattering.py:753-840,
                           MC/tools/singleScatter.py:205-239
  electron updates         MC/tools/electron.py:44-113
  direction update         MC/tools/rotation.py:41-53

Parity pins: tests/golden/gen_golden.py imports the reference itself (through
import stubs) and records its outputs; tests/test_oracle_golden.py checks this
module against them, including whole DS and continuous trajectories replayed
with the reference's own Python `random` stream.

Two random-number modes:
  * MTStream     - Python's `random` (MT19937) drawn in the reference's order,
                   channel list re-sorted by sigma each event (reference
                   behaviour, used to replay the reference exactly);
  * PhiloxStream - Philox4x32-10 keyed by the seed, counter (event, electron,
                   sim); slot 0 = channel, 1 = path length, 2 = polar angle
                   or table draw, 3 = azimuth; channels in fixed order.  This
                   is the stream the CUDA kernels use.
"""
import bisect
import math
import random

import numpy as np

# --------------------------------------------------------------------------
# constants (scipy.constants, CODATA 2022, as used by the reference)
# --------------------------------------------------------------------------
PI = math.pi
PI_EFOUR = 6.51408491409531e-14        # cm^2 eV^2, MC/tools/parameters.py:7
BOHR_R = 5.29177210544e-11             # m, MC/tools/parameters.py:8
AVOGADRO = 6.02214076e23
HBAR = 1.0545718176461565e-34
M_E = 9.1093837139e-31
E_CHARGE = 1.602176634e-19
EPS0 = 8.8541878188e-12

# per-species data, MC/tools/material.py:151-302
SPECIES = {
    "Al": dict(Z=13, n_val=3, E_val=72.55, density=2.70, atwt=26.98154,
               bethe_k=0.815, name_val="3s2-3p1",
               shells=[("1s", 1559.0, 2), ("2s", 118.0, 2), ("2p", 73.5, 6)]),
    "Si": dict(Z=14, n_val=4, E_val=99.42, density=2.33, atwt=28.085,
               bethe_k=0.822, name_val="3s2-3p2", xip_g=1360.0,
               shells=[("1s", 1189.0, 2), ("2s", 149.0, 2), ("2p", 100.0, 6)]),
    "Cu": dict(Z=29, n_val=11, E_val=75.1, density=8.96, atwt=63.546,
               bethe_k=0.83, name_val="3d10-4s2",
               shells=[("1s", 8980.0, 2), ("2s2p", 977.0, 8), ("3s", 120.0, 2),
                       ("3p", 74.0, 6)]),
    "Au": dict(Z=79, n_val=11, E_val=75.1, density=19.30, atwt=196.967,
               bethe_k=0.851, name_val="5d10-6s1",
               shells=[("2s2p", 12980.0, 8), ("3s3p3d", 2584.0, 18),
                       ("4s4p", 624.0, 8), ("4d", 341.0, 10), ("5s", 178.0, 2),
                       ("4f", 85.0, 14), ("5p2", 72.0, 2), ("5p4", 54.0, 4)]),
}

OUTCOMES = ("none", "bks", "abs", "trsm", "trdf", "long")
OUT_CODE = {name: i for i, name in enumerate(OUTCOMES)}


class Material:
    """Derived constants of one species (MC/tools/material.py:117-133)."""

    def __init__(self, species):
        p = SPECIES[species]
        self.species = species
        self.Z = p["Z"]
        self.n_val = p["n_val"]
        self.E_val = p["E_val"]
        self.bethe_k = p["bethe_k"]
        self.name_val = p["name_val"]
        self.shells = list(p["shells"])
        # extinction distance of the diffraction channel (material.py:225-226, Si only)
        self.xip_g = p.get("xip_g")
        # atomic number density in m^-3 (material.py:15-31)
        self.atnd = p["density"] * AVOGADRO / p["atwt"] * 1e6
        nv = self.n_val * self.atnd
        # plasmon and Fermi energies in eV (material.py:33-88)
        self.plasmon_e = HBAR * E_CHARGE * (nv / (EPS0 * M_E)) ** 0.5 / E_CHARGE
        self.fermi_e = HBAR ** 2 * (3.0 * PI ** 2 * nv) ** (2.0 / 3.0) / (2.0 * M_E) / E_CHARGE
        # mean ionisation energy of the Bethe law (stoppingPowers.py:134-137)
        Z = self.Z
        self.J = (9.76 * Z + 58.5 / Z ** 0.19) if Z >= 13 else 11.5 * Z

    @property
    def outer_shell(self):
        """The shell whose table samples every Gryzinski loss (scattering.py:625,
        probTables.py:579: tables['Gryz'][0] is the last entry of name_s)."""
        return self.shells[-1]


# --------------------------------------------------------------------------
# cross sections, stopping powers, dsigma/dW (scalar or numpy)
# --------------------------------------------------------------------------
def alpha(E, Z):
    """Rutherford screening, crossSections.py:14-27 (E in eV)."""
    return 3.4 * (Z ** 0.666667) / E


def ruther_sigma(E, Z):
    """crossSections.py:37-58, cm^2."""
    a = alpha(E, Z)
    Ek = E * 1e-3
    r = (Ek + 511.0) / (Ek + 1024.0)
    # r*r, not r**2: glibc's pow(x, 2) is not always correctly rounded, and
    # the C oracle's compiler folds pow(r, 2) to r*r
    return 5.21e-21 * (Z * Z / (Ek * Ek)) * (r * r) * (4.0 * PI) / (a * (1.0 + a))


def ruther_sigma_wDefl(E, Z):
    """crossSections.py:63-86: ruther_sigma with Z^2 -> Z (Z + 1)."""
    a = alpha(E, Z)
    Ek = E * 1e-3
    r = (Ek + 511.0) / (Ek + 1024.0)
    return 5.21e-21 * (Z * (Z + 1) / (Ek * Ek)) * (r * r) * (4.0 * PI) / (a * (1.0 + a))


def _nigram_beta(E, Z):
    """crossSections.py:108-112: 0.48 * 5.43 Z^(2/3) / E."""
    return 0.48 * (5.43 * Z ** (2.0 / 3.0) / E)


def ruther_N_sigma(E, Z):
    """crossSections.py:90-116 (Nigram screening), cm^2."""
    b = _nigram_beta(E, Z)
    return PI_EFOUR * (Z * Z) / (4.0 * b * (1.0 + b) * (E * E))


def ruther_N_sigma_wDefl(E, Z):
    """crossSections.py:120-147: ruther_N_sigma with Z^2 -> Z (Z + 1)."""
    b = _nigram_beta(E, Z)
    return PI_EFOUR * ((Z + 1) * Z) / (4.0 * b * (1.0 + b) * (E * E))


ELASTIC_MODELS = ("Ruth_vanilla", "Ruth_vanilla_wDefl", "Ruth_nigram", "Ruth_nigram_wDefl")


def elastic_sigma(model, E, Z):
    """The elastic total cross section of a resolved model name (the
    reference's string dispatch is resolved by the caller)."""
    if model == "Ruth_vanilla":
        return ruther_sigma(E, Z)
    if model == "Ruth_vanilla_wDefl":
        return ruther_sigma_wDefl(E, Z)
    if model == "Ruth_nigram":
        return ruther_N_sigma(E, Z)
    if model == "Ruth_nigram_wDefl":
        return ruther_N_sigma_wDefl(E, Z)
    raise ValueError(model)


def diffr_sigma(xip_g, n):
    """crossSections.py:329-349: 1 / (n xip_g) in units m^3/nm/cm^2 = 1e13, cm^2."""
    return 1.0 / (n * xip_g) * 1e13


def moller_sigma(E, Wc, nfree):
    """crossSections.py:183-208."""
    if E <= Wc:
        return 0.0
    eps = Wc * 1.0 / E
    return nfree * PI_EFOUR * (1.0 / (E * E)) * (1.0 / eps - 1.0 / (1.0 - eps) + math.log(eps / (1.0 - eps)))


def gryz_sigma(E, Esi, nsi):
    """crossSections.py:213-242."""
    if E <= Esi:
        return 0.0
    U = E * 1.0 / Esi
    return nsi * PI_EFOUR * ((U - 1.0) / (U + 1.0)) ** 1.5 * (
        1.0 + (2.0 * (1.0 - (1.0 / (2.0 * U))) / 3.0 * math.log(2.7 + ((U - 1.0) ** 0.5)))) / (E * Esi)


def quinn_sigma(E, Epl, Ef, n):
    """crossSections.py:247-284 (m^2 -> cm^2 is x1e4)."""
    if E <= Epl:
        return 0.0
    E_Ef = E * 1.0 / Ef
    Epl_Ef = Epl * 1.0 / Ef
    tot = Epl * math.log(((1.0 + Epl_Ef) ** 0.5 - 1.0) / (E_Ef ** 0.5 - (E_Ef - Epl_Ef) ** 0.5)) / (2.0 * BOHR_R * E)
    return tot / n * 1e4


def mfp_from_sigma(sigma, n):
    """scattering.py:19-36: 1/(n sigma) with m^3/cm^2/A = 1e14, in A."""
    return 1.0 / (n * sigma) * 1e14


def bethe_cl_sp(Z, E, n, J=None):
    """stoppingPowers.py:112-140, eV/A."""
    if J is None:
        J = (9.76 * Z + 58.5 / (Z ** 0.19)) if Z >= 13 else 11.5 * Z
    return 2.0 * PI_EFOUR * n * (Z / E) * math.log(1.166 * E / J) * 1e-14


def bethe_mod_sp_k(Z, E, n, k, J=None):
    """stoppingPowers.py:145-173 (Joy and Luo), eV/A."""
    if J is None:
        J = (9.76 * Z + 58.5 / (Z ** 0.19)) if Z >= 13 else 11.5 * Z
    return 2.0 * PI_EFOUR * n * (Z / E) * math.log(1.166 * (E + k * J) / J) * 1e-14


def bethe_mod_sp(E, n, Zi, Ei, Zval, Eval):
    """stoppingPowers.py:177-215 (explicit shells), eV/A."""
    pref = (2.0 * PI_EFOUR * n / E) * 1e-14
    s = Zval * math.log(E * 1.0 / Eval)
    for zi, eb in zip(Zi, Ei):
        s = s + zi * math.log(E * 1.0 / eb)
    return pref * s


def moller_dcs(E, W, nfree):
    """extFunctions.py:159-184 (numpy, float64)."""
    E = np.asarray(E, dtype=np.float64)
    W = np.asarray(W, dtype=np.float64)
    eps = W / E
    with np.errstate(divide="ignore", invalid="ignore"):
        v = nfree * PI_EFOUR * (1.0 / eps ** 2 + 1.0 / (1.0 - eps) ** 2 - 1.0 / (eps * (1.0 - eps))) / E ** 3
    return np.where(eps < 1.0, v, 0.0)


def gryz_dcs(E, W, nsi, Ebi):
    """extFunctions.py:189-219 (numpy, float64)."""
    E = np.asarray(E, dtype=np.float64)
    W = np.asarray(W, dtype=np.float64)
    eps = W / E
    epsB = Ebi / E
    with np.errstate(divide="ignore", invalid="ignore"):
        v = (nsi * PI_EFOUR * eps * (1.0 + epsB) ** (-1.5) * (1.0 - eps) ** (epsB / (epsB + eps))
             * ((1.0 - epsB) + 4.0 * epsB * np.log(2.7 + ((1.0 - eps) / epsB) ** 0.5) / (3.0 * eps)) / W ** 3)
    return np.where((eps < 1.0) & (epsB < 1.0), v, 0.0)


def maxW(E, Ef):
    """probTables.py:17-41: both Moller and Gryzinski use (E - Ef)/2."""
    return (E - Ef) * 0.5


def binary_coll_c2(E, W, Ef):
    """scattering.py:156-179: cos^2(theta/2), NaN when W > (E - Ef)/2."""
    if W <= maxW(E, Ef):
        return 0.5 * (math.sqrt(1.0 - W / E) + 1.0)
    return float("nan")


def rutherford_c2(E, Z, U):
    """scattering.py:125-152: cos^2(theta/2) = 1 - alpha U / (1 + alpha - U)."""
    a = alpha(E, Z)
    return 1.0 - (a * U / (1.0 + a - U))


# --------------------------------------------------------------------------
# CDF tables
# --------------------------------------------------------------------------
def table_cdf(kind, mat, Ws, Es):
    """Restates probTable.computeBlock (probTables.py:415-462) in float64.

    kind: 'Moller' or 'Gryz'.  Ws, Es are the float32 grids.  Returns
    (cdf64, valid): cdf64[nE, nW-1] is the normalised cumulative trapezoid
    sum, valid marks the intervals whose upper W edge is <= Wmax(E).  Stored
    tables keep float32(cdf64) where valid and 0 elsewhere (probTables.py:507);
    readers treat 0 as masked (probTables.py:533).
    """
    Ws32 = np.asarray(Ws, dtype=np.float32)
    Es32 = np.asarray(Es, dtype=np.float32)
    # the mask is evaluated in float32, as the reference's float32 meshes are
    wmax32 = ((Es32 - np.float32(mat.fermi_e)) * np.float32(0.5)).astype(np.float32)
    Wd = Ws32.astype(np.float64)
    Ed = Es32.astype(np.float64)[:, None]
    if kind == "Moller":
        f = moller_dcs(Ed, Wd[None, :], mat.n_val)
    else:
        _, Eb, ns = mat.outer_shell
        f = gryz_dcs(Ed, Wd[None, :], ns, Eb)
    dW = (Ws32[1:] - Ws32[:-1]).astype(np.float64)      # float32 differences
    steps = dW[None, :] * (f[:, :-1] + f[:, 1:]) / 2.0
    valid = Ws32[None, 1:] <= wmax32[:, None]
    steps = np.where(valid, steps, 0.0)
    cum = np.cumsum(steps, axis=1)
    tot = cum[:, -1:]
    with np.errstate(divide="ignore", invalid="ignore"):
        cdf = cum / tot
    return cdf, valid


def table_store32(cdf, valid):
    """The float32 table the reference writes to disk (masked -> 0)."""
    return np.where(valid, cdf, 0.0).astype(np.float32)


class Table:
    """A sampled table as the trajectory uses it: float32 grids promoted to
    float64 and the float32 CDF with zeros treated as +inf (masked)."""

    def __init__(self, Ws, Es, cdf32):
        self.Ws = np.asarray(Ws, dtype=np.float32).astype(np.float64)
        self.Es = np.asarray(Es, dtype=np.float32).astype(np.float64)
        c = np.asarray(cdf32, dtype=np.float32).astype(np.float64)
        self.cdf = np.where(c == 0.0, np.inf, c)
        self.Es_list = self.Es.tolist()
        self._rows = {}

    def row(self, i):
        r = self._rows.get(i)
        if r is None:
            r = self.cdf[i].tolist()
            self._rows[i] = r
        return r

    def pick(self, E, U):
        """scattering.py:63-94: upper-neighbour E row, lower W grid point."""
        i = bisect.bisect_left(self.Es_list, E)
        if i >= len(self.Es_list):
            i = len(self.Es_list) - 1
        j = bisect.bisect_left(self.row(i), U)
        if j >= self.Ws.size:
            j = self.Ws.size - 1
        return float(self.Ws[j]), i, j


# --------------------------------------------------------------------------
# random streams
# --------------------------------------------------------------------------
PHILOX_M0, PHILOX_M1 = 0xD2511F53, 0xCD9E8D57
PHILOX_W0, PHILOX_W1 = 0x9E3779B9, 0xBB67AE85
MASK32 = 0xFFFFFFFF


def philox4x32_10(ctr, key):
    """Philox4x32-10 (Salmon et al., SC'11), pure Python ints."""
    c0, c1, c2, c3 = (int(x) & MASK32 for x in ctr)
    k0, k1 = (int(x) & MASK32 for x in key)
    for r in range(10):
        if r:
            k0 = (k0 + PHILOX_W0) & MASK32
            k1 = (k1 + PHILOX_W1) & MASK32
        p0 = PHILOX_M0 * c0
        p1 = PHILOX_M1 * c2
        c0, c1, c2, c3 = ((p1 >> 32) ^ c1 ^ k0, p1 & MASK32, (p0 >> 32) ^ c3 ^ k1, p0 & MASK32)
    return c0, c1, c2, c3


def u32_to_unit(u):
    """(u + 1/2) / 2^32: a double in (0, 1), never 0 or 1."""
    return (u + 0.5) * 2.0 ** -32


class MTStream:
    """The reference's stream: random.random() drawn in call order."""

    sort_channels = True

    def __init__(self, seed):
        self.r = random.Random(seed)

    def begin_event(self, step):
        pass

    def u(self, slot):
        return self.r.random()


class PhiloxStream:
    """Counter-based stream: one Philox4x32-10 block per event."""

    sort_channels = False

    def __init__(self, seed, electron, sim=0):
        self.key = (seed & MASK32, (seed >> 32) & MASK32)
        self.elo = electron & MASK32
        self.ehi = (electron >> 32) & MASK32
        self.sim = sim & MASK32
        self.block = None

    def begin_event(self, step):
        self.block = philox4x32_10((step, self.elo, self.ehi, self.sim), self.key)

    def u(self, slot):
        return u32_to_unit(self.block[slot])


# --------------------------------------------------------------------------
# trajectories
# --------------------------------------------------------------------------
def beam_direction(s_tilt_deg):
    """multiScatter.py:97-100."""
    t = math.radians(s_tilt_deg)
    return [-math.sin(t), 0.0, math.cos(t)]


def _rotate(c2, half_phi, d, y):
    """electron.py:87-99 + rotation.py:41-53: q = q_az * q_pol applied to
    (d, y) through its rotation matrix, then each vector renormalised."""
    s_t = (1.0 - c2) ** 0.5
    c_t = c2 ** 0.5
    s_p = math.sin(half_phi)
    c_p = (1.0 - s_p * s_p) ** 0.5
    # q_pol = (c_t, y s_t), q_az = (c_p, d s_p)
    a1, b1, c1_, d1 = c_p, d[0] * s_p, d[1] * s_p, d[2] * s_p
    a2, b2, c2_, d2 = c_t, y[0] * s_t, y[1] * s_t, y[2] * s_t
    w = a1 * a2 - b1 * b2 - c1_ * c2_ - d1 * d2
    x = a1 * b2 + b1 * a2 + c1_ * d2 - d1 * c2_
    yy = a1 * c2_ - b1 * d2 + c1_ * a2 + d1 * b2
    z = a1 * d2 + b1 * c2_ - c1_ * b2 + d1 * a2
    n = w * w + x * x + yy * yy + z * z
    m = ((1.0 - 2.0 * (yy * yy + z * z) / n, 2.0 * (x * yy - z * w) / n, 2.0 * (x * z + yy * w) / n),
         (2.0 * (x * yy + z * w) / n, 1.0 - 2.0 * (x * x + z * z) / n, 2.0 * (yy * z - x * w) / n),
         (2.0 * (x * z - yy * w) / n, 2.0 * (yy * z + x * w) / n, 1.0 - 2.0 * (x * x + yy * yy) / n))
    out = []
    for v in (d, y):
        r = [m[i][0] * v[0] + m[i][1] * v[1] + m[i][2] * v[2] for i in range(3)]
        nn = math.sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2])
        out.append([r[0] / nn, r[1] / nn, r[2] / nn])
    return out[0], out[1]


class Electron:
    """State and output rows of one electron (electron.py:7-113)."""

    def __init__(self, E0, Emin, dir0, record=False):
        self.E = float(E0)
        self.Emin = float(Emin)
        self.pos = [0.0, 0.0, 0.0]
        self.dir = list(dir0)
        self.y = [0.0, 1.0, 0.0]
        self.outcome = None
        self.rows = []          # (outcome, final_E, dir, last_pos)
        self.events = [] if record else None
        self.steps = 0
        self.max_z = 0.0
        self.nan_events = 0
        self.diffracting = False

    def save(self):
        self.rows.append((self.outcome, self.E, list(self.dir), list(self.pos)))

    def update_xyz(self, s, maxz):
        """electron.py:64-84: leaving through the bottom face right after a
        diffraction event is 'trdf', otherwise 'trsm'."""
        p = [self.pos[i] + s * self.dir[i] for i in range(3)]
        if p[2] <= 0.0:
            self.outcome = "bks"
            self.save()
        elif p[2] >= maxz:
            self.outcome = "trdf" if self.diffracting else "trsm"
            self.save()
        else:
            self.pos = p
            if p[2] > self.max_z:
                self.max_z = p[2]

    def update_energy(self, W):
        """electron.py:44-59: the 'abs' row keeps the pre-loss energy."""
        e = self.E - W
        if e <= self.Emin:
            self.outcome = "abs"
            self.save()
        self.E = e

    def update_direction(self, c2, half_phi):
        self.dir, self.y = _rotate(c2, half_phi, self.dir, self.y)


CH_RUTH, CH_MOLLER, CH_QUINN, CH_GRYZ0, CH_DIFF = 0, 1, 2, 3, 11


def channel_names(mat):
    """Channel codes -> reference type labels (scattering.py:483-516)."""
    names = ["Ruth", "Moller", "Quinn"] + ["Gryz" + s[0] for s in mat.shells]
    names += [""] * (CH_DIFF - len(names)) + ["diff"]
    return names


def ds_sigmas(E, mat, Wc, elastic="Ruth_vanilla", diff=False):
    """scattering.py:483-516 in the reference's insertion order, as
    (code, sigma) pairs: Ruth, Moller, Gryz<shell> in name_s order, Quinn,
    then the diffraction channel when diffMFP is on."""
    out = [(CH_RUTH, elastic_sigma(elastic, E, mat.Z)), (CH_MOLLER, moller_sigma(E, Wc, mat.n_val))]
    for k, (_, Es, ns) in enumerate(mat.shells):
        out.append((CH_GRYZ0 + k, gryz_sigma(E, Es, ns)))
    out.append((CH_QUINN, quinn_sigma(E, mat.plasmon_e, mat.fermi_e, mat.atnd)))
    if diff:
        out.append((CH_DIFF, diffr_sigma(mat.xip_g, mat.atnd)))
    return out


def pick_channel(sig, U, sort_channels):
    """scattering.py:39-59: bisect_left over cumulative sigma / total."""
    if sort_channels:
        sig = sorted(sig, key=lambda t: t[1], reverse=True)
    tot = 0.0
    for _, s in sig:
        tot += s
    cum = 0.0
    probs = []
    for _, s in sig:
        cum += s
        probs.append(cum / tot)
    i = bisect.bisect_left(probs, U)
    return sig[min(i, len(sig) - 1)][0]


def trajectory_ds(el, mat, Wc, maxScatt, maxz, tables, rng, elastic="Ruth_vanilla", diff=False):
    """singleScatter.py:10-41 with scatter_discrete (scattering.py:440-679).

    tables = (moller Table, gryz Table for the outermost shell).  With diff
    (diffMFP) a diffraction event steps with mean free path xip_g
    (scattering.py:540-548), loses nothing and keeps its direction
    (:658-668), and marks the electron diffracting for the exit test."""
    t_m, t_g = tables
    num = 0
    while el.outcome not in ("abs", "bks", "trsm", "trdf", "long"):
        Ei = el.E
        sig = ds_sigmas(Ei, mat, Wc, elastic, diff)
        stot = 0.0
        for _, s in sig:
            stot += s
        mfp = mfp_from_sigma(stot, mat.atnd)
        pos0 = list(el.pos)
        num += 1
        if num > maxScatt:
            el.outcome = "long"
            el.save()
            return
        rng.begin_event(num - 1)
        ch = pick_channel(sig, rng.u(0), rng.sort_channels)
        if ch == CH_DIFF:
            mfp = mat.xip_g
        el.diffracting = ch == CH_DIFF
        s = -mfp * math.log(rng.u(1))
        el.update_xyz(s, maxz)
        if ch == CH_DIFF:
            W = 0.0
            c2 = 1.0
        elif ch == CH_RUTH:
            W = 0.0
            c2 = rutherford_c2(Ei, mat.Z, rng.u(2))
        elif ch == CH_MOLLER:
            W, _, _ = t_m.pick(Ei, rng.u(2))
            c2 = binary_coll_c2(Ei, W, mat.fermi_e)
        elif ch == CH_QUINN:
            W = mat.plasmon_e
            c2 = 1.0
        else:
            W, _, _ = t_g.pick(Ei, rng.u(2))
            c2 = binary_coll_c2(Ei, W, mat.fermi_e)
        if c2 != c2:
            el.nan_events += 1
        half_phi = PI * rng.u(3)
        el.update_energy(W)
        if el.events is not None:
            el.events.append((ch, Ei, W, c2, half_phi, s, pos0[0], pos0[1], pos0[2], el.E))
        el.update_direction(c2, half_phi)
        el.steps = num


def stopping_power(model, mat, E, J=None, n=None):
    """Continuous-mode energy-loss law; JL and explicit use the law the
    reference names (the reference itself calls the classical one)."""
    n = mat.atnd if n is None else n
    if model == "classical":
        return bethe_cl_sp(mat.Z, E, n, J)
    if model == "JL":
        return bethe_mod_sp_k(mat.Z, E, n, mat.bethe_k, J)
    if model == "explicit":
        return bethe_mod_sp(E, n, [s[2] for s in mat.shells], [s[1] for s in mat.shells],
                            mat.n_val, mat.E_val)
    raise ValueError(model)


class ContStatus:
    def __init__(self):
        self.long_path = 0      # s >= 1e4 A (scattering.py:809 asserts)
        self.clamped = 0        # dE >= E (scattering.py:822 asserts)


def trajectory_cont(el, mat, maxScatt, maxz, model, rng, status=None, J=None, n=None, elastic="Ruth_vanilla"):
    """singleScatter.py:205-239 with scatter_continuous_* (scattering.py:753-883).

    maxz is passed (the reference's caller omits it); an energy loss >= E is
    clamped to E and counted instead of aborting the job."""
    n_at = mat.atnd if n is None else n
    num = 0
    while el.outcome not in ("abs", "bks", "trsm"):
        Ei = el.E
        mfp = mfp_from_sigma(elastic_sigma(elastic, Ei, mat.Z), n_at)
        pos0 = list(el.pos)
        num += 1
        if num > maxScatt:
            el.outcome = "long"
            el.save()
            return
        rng.begin_event(num - 1)
        s = -mfp * math.log(rng.u(1))
        if status is not None and not s < 1e4:
            status.long_path += 1
        el.update_xyz(s, maxz)
        dE = s * stopping_power(model, mat, Ei, J, n_at)
        if not dE < Ei:
            if status is not None:
                status.clamped += 1
            dE = Ei
        el.update_energy(dE)
        c2 = rutherford_c2(Ei, mat.Z, rng.u(2))
        half_phi = PI * rng.u(3)
        if el.events is not None:
            el.events.append((CH_RUTH, Ei, dE, c2, half_phi, s, pos0[0], pos0[1], pos0[2], el.E))
        el.update_direction(c2, half_phi)
        el.steps = num


def run_ds(mat, E0, Emin, s_tilt, Wc, maxScatt, maxz, tables, n_el, seed, sim=0,
           first=0, record=False, elastic="Ruth_vanilla", diff=False):
    """One DS simulation on the Philox stream; returns the Electron objects."""
    d0 = beam_direction(s_tilt)
    out = []
    for k in range(first, first + n_el):
        el = Electron(E0, Emin, d0, record)
        trajectory_ds(el, mat, Wc, maxScatt, maxz, tables, PhiloxStream(seed, k, sim), elastic, diff)
        out.append(el)
    return out


def run_cont(mat, E0, Emin, s_tilt, maxScatt, maxz, model, n_el, seed, sim=0, first=0,
             record=False, J=None, n=None, status=None, elastic="Ruth_vanilla"):
    d0 = beam_direction(s_tilt)
    out = []
    for k in range(first, first + n_el):
        el = Electron(E0, Emin, d0, record)
        trajectory_cont(el, mat, maxScatt, maxz, model, PhiloxStream(seed, k, sim), status, J, n, elastic)
        out.append(el)
    return out


# --------------------------------------------------------------------------
# detector projection
# --------------------------------------------------------------------------
def proj_on_detector(xyz_exit, alpha, xy_PC, L):
    """rotation.py:78-102: rotate each direction by conj(q_SD), q_SD =
    (cos(alpha/2), sin(alpha/2), 0, 0), through the rotation matrix of a
    quaternion (entries / |q|^2, as numpy-quaternion's rotate_vectors),
    subtract t = (x_PC, y_PC, L), keep x and y.  Returns an (n, 2) array."""
    c = math.cos(math.radians(alpha) / 2.0)
    s = (1.0 - c * c) ** 0.5
    w, x, y, z = c, -s, 0.0, 0.0
    n = w * w + x * x + y * y + z * z
    m = np.array([
        [1.0 - 2.0 * (y * y + z * z) / n, 2.0 * (x * y - z * w) / n, 2.0 * (x * z + y * w) / n],
        [2.0 * (x * y + z * w) / n, 1.0 - 2.0 * (x * x + z * z) / n, 2.0 * (y * z - x * w) / n],
        [2.0 * (x * z - y * w) / n, 2.0 * (y * z + x * w) / n, 1.0 - 2.0 * (x * x + y * y) / n],
    ])
    v = np.asarray(xyz_exit, dtype=np.float64).reshape(-1, 3)
    t = np.array([xy_PC[0], xy_PC[1], L], dtype=np.float64)
    return (v @ m.T - t)[:, 0:2]


# --------------------------------------------------------------------------
# theory distributions and the two-sample test of the reference's tests
# --------------------------------------------------------------------------
def ruth_theta_ppf(x, E, Z):
    """distributions.py:400-416 (Ruth_diffCS_E._ppf): polar angle in degrees
    of the Rutherford distribution at energy E for uniform x."""
    a = alpha(np.asarray(E, dtype=np.float64), Z)
    x = np.asarray(x, dtype=np.float64)
    return np.degrees(np.arccos(1.0 - (2.0 * a * x) / (1.0 + a - x)))


def theory_W_cdf(kind, mat, E, Wmin, npts=20001):
    """distributions.py:21-124: CDF of the energy loss at energy E from
    dsigma/dW between Wmin and maxW(E) (Moller: valence electrons; Gryz: the
    outermost shell, Wmin its binding energy).  Integrated on a geometric W
    grid by the trapezoid rule in ln W; returns (W grid, CDF)."""
    Wmax = maxW(E, mat.fermi_e)
    W = np.geomspace(Wmin, Wmax, npts)
    if kind == "Moller":
        f = moller_dcs(E, W, mat.n_val)
    else:
        _, Eb, ns = mat.outer_shell
        f = gryz_dcs(E, W, ns, Eb)
    g = f * W
    c = np.concatenate([[0.0], np.cumsum(0.5 * (g[1:] + g[:-1]) * np.diff(np.log(W)))])
    return W, c / c[-1]


def theory_W_sample(kind, mat, E, Wmin, u, npts=20001):
    """Inverse-CDF samples of the energy loss at energy E for uniforms u."""
    W, c = theory_W_cdf(kind, mat, E, Wmin, npts)
    return np.interp(np.asarray(u, dtype=np.float64), c, W)


def theta_from_c2(c2):
    """tests/testThings.py:153-161: degrees from cos^2(theta/2)."""
    return np.degrees(2.0 * np.arccos(np.asarray(c2, dtype=np.float64) ** 0.5))


def watson_u2(x, y):
    """Two-sample Watson U^2 as tests/testThings.py:255-316 computes it
    (Mardia and Jupp, Directional Statistics, eq. 8.3.7): over the sorted
    unique pooled values, d_k = F_x - F_y, U^2 = nx ny (sum d^2 - (sum d)^2
    / N) / N^2."""
    x = np.sort(np.asarray(x, dtype=np.float64))
    y = np.sort(np.asarray(y, dtype=np.float64))
    nx, ny = x.size, y.size
    N = nx + ny
    t = np.unique(np.concatenate([x, y]))
    d = np.searchsorted(x, t, side="right") / nx - np.searchsorted(y, t, side="right") / ny
    return nx * ny * (np.sum(d * d) - np.sum(d) ** 2 / N) / N ** 2


def watson_u2_pvalue(u2, terms=50):
    """Asymptotic upper tail of U^2: 2 sum_k (-1)^(k-1) exp(-2 k^2 pi^2 u)
    (the reference's critical value 0.152 is its 10% point)."""
    if u2 <= 1e-4:        # the alternating series needs more terms there; the tail is 1
        return 1.0
    k = np.arange(1, terms + 1)
    return float(min(1.0, max(0.0, 2.0 * np.sum((-1.0) ** (k - 1) * np.exp(-2.0 * k * k * PI * PI * u2)))))

