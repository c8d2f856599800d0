"""Shared helpers of the GPU tests: run the CUDA path and the C oracle on the
same inputs (same Philox stream, same tables copied back from the GPU)."""
import math

import numpy as np

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


def run_pair(p, n, seed=1, precision="fp64", nthreads=None):
    """GPU run and C-oracle run of the same n electrons."""
    g = engine.run(p, num_el=n, seed=seed, precision=precision)
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
