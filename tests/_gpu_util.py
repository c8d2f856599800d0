"""Shared helpers of the GPU tests: run the CUDA path and the C oracle on the
same inputs (same Philox stream, same tables copied back from the GPU)."""
import math
import os

import numpy as np
from scipy import stats

import coracle
import mcd_oracle as O
from mcd import _lib, engine, tables

GOLDEN_TABLES = {
    # table-config name -> (species, E0, Emin, Wc, tol)
    "cfg1": ("Si", 10000.0, 1000.0, 100.0, 1e-3),
    "cfg3": ("Au", 30000.0, 500.0, 50.0, 1e-4),
    "cfg4_Al_5": ("Al", 5000.0, 1000.0, 100.0, 1e-3),
    "cfg4_Cu_20": ("Cu", 20000.0, 1000.0, 100.0, 1e-3),
    "cfg4_Au_30": ("Au", 30000.0, 1000.0, 100.0, 1e-3),
}


def input_par(species, E0, Emin, tilt, Wc=100.0, tol=1e-3, mode="DS", bethe="classical", elastic="Ruth_vanilla",
              diffMFP=False, thickness=1e30):
    return dict(material=species, E0=E0, Emin=Emin, s_tilt=tilt, Wc=Wc, tol_E=tol, tol_W=tol, mode=mode,
                Bethe_model=bethe, num_el=0, elastic=elastic, diffMFP=diffMFP, thickness=thickness)


ELASTIC_NAME = {v: k for k, v in _lib.ELASTIC.items()}


def gpu_tables(p):
    mat = _lib.material(p["material"])
    return tables.ds_tables(mat, p["E0"], p["Emin"], p["Wc"], p["tol_E"], p["tol_W"])


def host_copies(dev_tables):
    out = []
    for t in dev_tables:
        out.append(coracle.HostTable(t.Ws.cpu().numpy(), t.Es.cpu().numpy(), t.cdf.cpu().numpy()))
    return out


def run_pair(p, n, seed=1, precision="fp64", nthreads=None, tabulated=False):
    """GPU run and C-oracle run of the same n electrons (tabulated: the GPU
    reads the simulation's cross-section table for its precision)."""
    g = engine.run(p, num_el=n, seed=seed, precision=precision, tabulated=tabulated)
    mat = O.Material(p["material"])
    ds = "DS" in p["mode"]
    ht = host_copies(gpu_tables(p)) if ds else None
    sim = engine.make_sim(p, n)
    c = coracle.run(mat, p["E0"], p["Emin"], p["s_tilt"], n, seed=seed, mode="DS" if ds else "cont",
                    Wc=p["Wc"], tables=ht, bethe=p.get("Bethe_model", "classical"), nthreads=nthreads,
                    elastic=ELASTIC_NAME[sim.elastic], diff=bool(sim.diff_mfp), thickness=sim.thickness)
    return g, c


def eta_z(n1, k1, n2, k2):
    p = (k1 + k2) / (n1 + n2)
    if p in (0.0, 1.0):
        return 0.0
    s = math.sqrt(p * (1 - p) * (1.0 / n1 + 1.0 / n2))
    return abs(k1 / n1 - k2 / n2) / s


def theta_deg(c2):
    c2 = np.clip(np.asarray(c2, dtype=np.float64), 0.0, 1.0)
    return np.degrees(2.0 * np.arccos(np.sqrt(c2)))


# ---------------------------------------------------------------------------
# the three FP32 DS code paths the statistical tests pin to the reference
# ---------------------------------------------------------------------------
# plain_inline     one launch, every cross section evaluated per event
# plain_tabulated  one launch reading the simulation's cross-section table
# batched          the benchmarked configuration: the persistent kernel with
#                  the tables mcd_batch_prepare builds, in the shape the
#                  benchmark's autotuner picks on the 64-simulation workload
#                  (two blocks of 576 per SM at 56 registers, tune variant
#                  bit 0; refill 1); one simulation with sim id 0, so it draws
#                  the same Philox words as the plain launches (the results
#                  do not depend on the shape: tests/test_gpu_batched.py)
VARIANTS = ("plain_inline", "plain_tabulated", "batched")
BENCH_TUNE = (576, 0, 1, 1, 0)


def run_variant(variant, p, n, seed, electrons=True, ring_capacity=0, ring_fields=0):
    """One FP32 run of n electrons of p on a code path of VARIANTS."""
    if variant in ("plain_inline", "plain_tabulated"):
        return engine.run(p, num_el=n, seed=seed, precision="fp32", electrons=electrons,
                          ring_capacity=ring_capacity, ring_fields=ring_fields,
                          tabulated=variant == "plain_tabulated")
    if variant != "batched":
        raise ValueError(variant)
    b = engine.Batch([dict(p, num_el=n)], seed=seed, electrons=electrons)
    tune = _lib.Tune(*BENCH_TUNE)
    events, total = None, 0
    if ring_capacity:
        tallies, status, events, total = b.run_events(ring_capacity, fields=ring_fields, tune=tune)
    else:
        tallies, status = b.run(tune)
    rows = b.electrons(0) if electrons else None
    return engine.RunResult(tallies[0], status, rows, events, total)


# ---------------------------------------------------------------------------
# a rule for many independent tests at the p > 0.01 level
# ---------------------------------------------------------------------------
P_MIN = 0.01
K_SUB = 10


def max_rejections(k=K_SUB, p=P_MIN, q=0.999):
    """The 99.9% quantile of Binomial(k, p): with no real difference, more
    than this many of k independent tests at level p reject with probability
    below 1e-3 (k = 10, p = 0.01: 2)."""
    return int(stats.binom.ppf(q, k, p))


def assert_subsamples(pvalues, what=""):
    """K independent subsamples, each tested at p > P_MIN: fail when more of
    them reject than chance allows (max_rejections)."""
    pv = [float(x) for x in pvalues]
    bad = sum(x <= P_MIN for x in pv)
    assert bad <= max_rejections(len(pv)), (what, bad, ["%.3g" % x for x in pv])


# ---------------------------------------------------------------------------
# oracle tables on the reference's own grids (tests/golden/tables.npz)
# ---------------------------------------------------------------------------
GOLDEN_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def oracle_tables_from_golden(key):
    """The oracle's FP64-filled tables (stored as float32, as the reference
    stores them) on the W/E grids the reference's grid search chose for
    table configuration `key` (e.g. 'cfg4_Al_5')."""
    T = np.load(os.path.join(GOLDEN_DIR, "tables.npz"))
    sp = str(T[key + "/Moller/species"])
    mat = O.Material(sp)
    return mat, [coracle.HostTable.build(kind, mat, T["%s/%s/Ws" % (key, kind)], T["%s/%s/Es" % (key, kind)])
                 for kind in ("Moller", "Gryz")]
