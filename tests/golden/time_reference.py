"""Time the reference's own Python code where it is installed, and write
tests/golden/reference_timing.json (committed; bench.py carries it in its
line as `reference_python`, because the GPU host has no copy of the
reference).

    MCD_REFERENCE_ROOT=<reference checkout> python tests/golden/time_reference.py

What is timed, all through the reference's modules (tests/golden/refload.py
supplies stubs for its missing third-party imports):
  tables   the table build of every (material, E0) pair of the 64-simulation
           workload and of the Au 30 keV tol 1e-4 configuration, one probTable
           per sampled table: set_Ws + set_Es (the grid search), then
           computeBlock + mapToMemory + readFromMemory (the fill), i.e. the
           work genTables does per table (MC/tools/probTables.py:541-614)
  worker   multiTraj_DS (MC/tools/multiScatter.py:66-116) in jobs of 4
           electrons (MC/doScatter.py:216) with the default input.file
           outputs (electron: outcome, final_E, final_dir, last_pos;
           scatter: type, position, energy), in a fork pool of 1 worker and of
           one worker per host core (MC/doScatter.py:46, 87-94): the Si
           10 keV configuration (1000 electrons on all cores, 200 on one) and
           a num_el-weighted sample of the 64-simulation workload.
Results are gathered in memory; the HDF5 writer is left out (pandas and
PyTables are absent).
"""
import json
import multiprocessing as mp
import os
import platform
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import gen_golden as G  # noqa: E402

sys.path.insert(0, ROOT)
import bench  # noqa: E402  (the workload definition only)

EL_COLS = ["outcome", "final_E", "final_dir", "last_pos"]
SC_COLS = ["type", "position", "energy"]
PER_JOB = 4
_CTX = {}


def time_tables():
    out = {}
    pairs = sorted({(s["material"], s["E0"]) for s in bench.workload()})
    total = 0.0
    for sp, E0 in pairs:
        rec = {}
        for kind in ("Moller", "Gryz"):
            t0 = time.perf_counter()
            tb, _ = G.build_table(kind, sp, E0, 1000.0, 100.0, 1e-3)
            rec[kind] = {"s": time.perf_counter() - t0, "nE": int(len(tb.Es)), "nW": int(len(tb.Ws))}
        out["%s_%d" % (sp, int(E0 / 1000))] = rec
        total += rec["Moller"]["s"] + rec["Gryz"]["s"]
        print(sp, E0, rec, flush=True)
    au = {}
    for kind in ("Moller", "Gryz"):
        t0 = time.perf_counter()
        tb, _ = G.build_table(kind, "Au", 30000.0, 500.0, 50.0, 1e-4)
        au[kind] = {"s": time.perf_counter() - t0, "nE": int(len(tb.Es)), "nW": int(len(tb.Ws))}
    print("Au tol 1e-4", au, flush=True)
    return {"workload_pairs": out, "workload_total_s": total,
            "au30_tol1e-4": au, "au30_tol1e-4_total_s": au["Moller"]["s"] + au["Gryz"]["s"]}


def _job(j):
    c = _CTX[j[0]]
    m = G._load()
    ip = dict(E0=c["E0"], Emin=c["Emin"], s_tilt=c["tilt"], Wc=c["Wc"], maxScatt=G.BIG_MAXSCATT,
              thickness=G.INF_Z, elastic="Ruth_vanilla", diffMFP=False)
    with np.errstate(invalid="ignore"):
        res = m["multiScatter"].multiTraj_DS(ip, j[1], c["mat"], c["tables"],
                                             {"el_output": EL_COLS, "scat_output": SC_COLS})
    return sum(len(r["scats"]["type"]) for r in res), len(res)


def run_pool(jobs, workers):
    t0 = time.perf_counter()
    with mp.get_context("fork").Pool(workers) as pool:
        out = pool.map(_job, jobs, chunksize=1)
    dt = time.perf_counter() - t0
    ev = sum(e for e, _ in out)
    el = sum(n for _, n in out)
    return {"workers": workers, "electrons": el, "events": ev, "wall_s": dt, "events_per_s": ev / dt,
            "electrons_per_s": el / dt}


def prepare(key, sp, E0, Emin, Wc, tol, tilt):
    tables, mat = G.ds_tables((key, sp, E0, Emin, Wc, tol))
    _CTX[key] = dict(mat=mat, tables=tables, E0=E0, Emin=Emin, Wc=Wc, tilt=tilt)


def jobs_for(key, n):
    return [(key, min(PER_JOB, n - k)) for k in range(0, n, PER_JOB)]


def time_worker():
    cores = os.cpu_count() or 1
    out = {}
    prepare("si10", "Si", 10000.0, 1000.0, 100.0, 1e-3, 0.0)
    out["si10_1000el"] = {"config": "DS Si, E0 10 keV, Emin 1 keV, tilt 0, Wc 100 eV, tol 1e-3",
                          "all_cores": run_pool(jobs_for("si10", 1000), cores),
                          "one_core": run_pool(jobs_for("si10", 200), 1)}
    print("si10", out["si10_1000el"], flush=True)
    # the 64-simulation workload, num_el-weighted (at least one electron each)
    sims = bench.workload()
    sizes = bench.sample_sizes(sims, 400)
    jobs = []
    for k, (s, n) in enumerate(zip(sims, sizes)):
        key = "w%d" % k
        prepare(key, s["material"], s["E0"], s["Emin"], s["Wc"], s["tol_E"], s["s_tilt"])
        jobs += jobs_for(key, n)
    jobs.sort(key=lambda j: -_CTX[j[0]]["E0"])     # long trajectories first
    out["workload_sample"] = {"config": bench.WORKLOAD_NAME,
                              "sample": "num_el-weighted, %d electrons" % sum(sizes),
                              "all_cores": run_pool(jobs, cores)}
    print("workload", out["workload_sample"], flush=True)
    one = [j for j in jobs if int(j[0][1:]) % 4 == 0]
    out["workload_sample"]["one_core"] = run_pool(one, 1)
    out["workload_sample"]["one_core"]["sample"] = "the tilt-0 simulations of the sample above"
    print("workload 1 core", out["workload_sample"]["one_core"], flush=True)
    return out


def main():
    rec = {"what": "the reference's own Python (MC-discrete) run here through import stubs",
           "host": {"machine": platform.machine(), "processor": platform.processor() or platform.machine(),
                    "cores": os.cpu_count(), "python": platform.python_version(), "numpy": np.__version__},
           "date": time.strftime("%Y-%m-%d")}
    G._load()
    rec["tables"] = time_tables()
    rec["worker"] = time_worker()
    with open(os.path.join(HERE, "reference_timing.json"), "w") as f:
        json.dump(rec, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    main()
