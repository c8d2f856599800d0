"""Generate the golden fixtures in tests/golden/ from the reference itself.

Runs only where a checkout of the reference exists, named by the
MCD_REFERENCE_ROOT environment variable; the fixtures it writes are
committed and the tests read those, so nothing on the GPU host needs the
reference.  Usage:

    MCD_REFERENCE_ROOT=<checkout> python tests/golden/gen_golden.py physics tables replay   # seconds
    MCD_REFERENCE_ROOT=<checkout> python tests/golden/gen_golden.py stats                   # minutes

Parts:
  physics  material constants, total cross sections, stopping powers,
           dsigma/dW, binary-collision and Rutherford angles
  tables   W/E grids chosen by the reference's own grid search and the CDF
           tables of probTable.computeBlock, mapToMemory and readFromMemory,
           for every table the benchmark configurations sample
  replay   whole DS and continuous trajectories of the reference driven by a
           seeded Python `random` stream (for exact replay by the oracle)
  stats    large DS samples of the reference (outcomes, exit energies and
           directions, first-event channel mix, per-channel samples)

Deliberate choices, each forced by running the reference here:
  * Under NumPy 2 a float32 table value silently turns the reference's
    electron energy into float32 after the first table event (NEP 50).  The
    author ran NumPy 1.x, where it stays float64.  The replay and stats parts
    therefore hold the float32 grids and tables as float64 arrays with the
    same values, which restores the NumPy 1.x dtype flow.
  * The reference reseeds Python `random` with pid * int(time()) at every job
    (MC/tools/multiScatter.py:94), so two jobs a worker starts within the same
    second repeat the same trajectories.  The stats part drives the same
    per-electron calls as multiTraj_DS (electron + trajectory_DS) with one
    distinct seed per job instead.
  * Continuous mode cannot run through multiTraj_cont (argument mismatch,
    MC/tools/multiScatter.py:206-207 vs MC/tools/singleScatter.py:205); the
    replay part runs the loop of trajectory_cont_cl with maxz passed.
"""
import multiprocessing as mp
import os
import random
import sys
import time

import numpy as np
import numpy.ma as ma

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
import refload  # noqa: E402

M = None  # reference modules, filled by _load()

SPECIES = ("Al", "Si", "Cu", "Au")
BIG_MAXSCATT = 10 ** 9
INF_Z = 1e30

# table configurations: (name, species, E0, Emin, Wc, tol)
CFG1 = ("cfg1", "Si", 10000.0, 1000.0, 100.0, 1e-3)
CFG3 = ("cfg3", "Au", 30000.0, 500.0, 50.0, 1e-4)
CFG4 = [("cfg4_%s_%d" % (sp, int(E0 / 1000)), sp, E0, 1000.0, 100.0, 1e-3)
        for sp in SPECIES for E0 in (5000.0, 10000.0, 20000.0, 30000.0)]


def _load():
    global M
    if M is None:
        M, _ = refload.load()
    return M


# ---------------------------------------------------------------------------
def part_physics():
    m = _load()
    cs, sp, ef, sc, pt = m["crossSections"], m["stoppingPowers"], m["extFunctions"], m["scattering"], m["probTables"]
    out = {}
    Egrid = np.concatenate([np.geomspace(60.0, 30000.0, 37), [99.9, 100.0, 100.1, 1000.0, 1189.0, 1190.0,
                                                              10000.0, 20000.0, 30000.0]])
    out["E"] = Egrid
    for spc in SPECIES:
        mat = m["material"].material(spc)
        p = mat.params
        out[spc + "/const"] = np.array([mat.atnd, mat.plasmon_e, mat.fermi_e])
        out[spc + "/alpha"] = np.array([cs.alpha(E, p["Z"]) for E in Egrid])
        out[spc + "/ruth"] = np.array([cs.ruther_sigma(E, p["Z"]) for E in Egrid])
        out[spc + "/ruth_wdefl"] = np.array([cs.ruther_sigma_wDefl(E, p["Z"]) for E in Egrid])
        out[spc + "/ruth_nigram"] = np.array([cs.ruther_N_sigma(E, p["Z"]) for E in Egrid])
        out[spc + "/ruth_nigram_wdefl"] = np.array([cs.ruther_N_sigma_wDefl(E, p["Z"]) for E in Egrid])
        if "xip_g" in p:
            out[spc + "/xip_g"] = np.array(float(p["xip_g"]))
            out[spc + "/diffr"] = np.array(cs.diffr_sigma(p["xip_g"], mat.atnd, 0.0))
        for Wc in (10.0, 50.0, 100.0):
            out[spc + "/moller/%g" % Wc] = np.array([cs.moller_sigma(E, Wc, p["n_val"]) for E in Egrid])
        for sh in p["name_s"]:
            out[spc + "/gryz/" + sh] = np.array([cs.gryz_sigma(E, p["Es"][sh], p["ns"][sh]) for E in Egrid])
        Eq = Egrid[Egrid > mat.plasmon_e]
        out[spc + "/quinn_E"] = Eq
        out[spc + "/quinn"] = np.array([cs.quinn_sigma(E, mat.plasmon_e, mat.fermi_e, mat.atnd) for E in Eq])
        Eb = Egrid[Egrid > 300.0]
        out[spc + "/bethe_E"] = Eb
        out[spc + "/bethe_cl"] = np.array([sp.bethe_cl_sp(p["Z"], E, mat.atnd) for E in Eb])
        out[spc + "/bethe_jl"] = np.array([sp.bethe_mod_sp_k(p["Z"], E, mat.atnd, p["bethe_k"]) for E in Eb])
        Zi = [p["ns"][s] for s in p["name_s"]]
        Ei = [p["Es"][s] for s in p["name_s"]]
        out[spc + "/bethe_ex"] = np.array([sp.bethe_mod_sp(E, mat.atnd, Zi, Ei, p["n_val"], p["E_val"]) for E in Eb])
        tot = np.array([cs.ruther_sigma(E, p["Z"]) + cs.moller_sigma(E, 100.0, p["n_val"]) for E in Egrid])
        out[spc + "/mfp"] = np.array([sc.mfp_from_sigma(t, mat.atnd) for t in tot])
        # dsigma/dW on an (E, W) grid of float64 values
        Ed = np.array([500.0, 1000.0, 5000.0, 20000.0])
        Wd = np.geomspace(11.0, 9000.0, 25)
        EE, WW = np.meshgrid(Ed, Wd, indexing="ij")
        out[spc + "/dcs_E"], out[spc + "/dcs_W"] = EE, WW
        out[spc + "/moller_dcs"] = np.asarray(ef.moller_dCS(EE, WW, p["n_val"]), dtype=np.float64)
        sh = p["name_s"][-1]
        out[spc + "/gryz_dcs"] = np.asarray(ef.gryz_dCS(EE, WW, p["ns"][sh], p["Es"][sh]), dtype=np.float64)
        out[spc + "/maxW"] = np.array([pt.maxW_moller(E, mat.fermi_e) for E in Ed])
        # binary collision model and Rutherford polar angle
        Ws = np.array([0.0, 10.0, 100.0, 400.0, 499.0, 2000.0, 4990.0, 5000.0])
        out[spc + "/bc_W"] = Ws
        with np.errstate(invalid="ignore"):
            out[spc + "/bc"] = np.array([[float(sc.binaryCollModel(E, W, mat.fermi_e)) for W in Ws] for E in Ed])
        us, c2 = [], []
        for k in range(64):
            random.seed(7000 + k)
            u = random.random()
            random.seed(7000 + k)
            E = float(Egrid[k % len(Egrid)])
            us.append((E, u))
            c2.append(sc.Rutherford_halfPol(E, p["Z"]))
        out[spc + "/ruth_EU"] = np.array(us)
        out[spc + "/ruth_c2"] = np.array(c2)
    # detector projection (MC/tools/rotation.py:78-102) of seeded unit
    # directions and the axes, at the geometry of MC/tools/parameters.py:22-33
    # and at other tilts
    rng = np.random.default_rng(11)
    d = rng.normal(size=(61, 3))
    d = np.vstack([d / np.linalg.norm(d, axis=1)[:, None], np.eye(3), -np.eye(3)])
    xy_pc = np.asarray(m["parameters"].xy_PC, dtype=np.float64)
    out["det/dirs"] = d
    out["det/xy_PC"] = xy_pc
    out["det/L"] = np.array(float(m["parameters"].L))
    out["det/alphas"] = np.array([float(m["parameters"].alpha), 0.0, 45.0, 70.0, 90.0, 180.0])
    for a in out["det/alphas"]:
        res = m["rotation"].projOnDetector(list(d), a, xy_pc, out["det/L"])
        out["det/xy/%g" % a] = np.asarray(res, dtype=np.float64)
    np.savez_compressed(os.path.join(HERE, "physics.npz"), **out)
    print("physics.npz:", len(out), "arrays")


# ---------------------------------------------------------------------------
def build_table(kind, species, E0, Emin, Wc, tol):
    """Build one table through the reference's own methods."""
    m = _load()
    pt, ef = m["probTables"], m["extFunctions"]
    mat = m["material"].material(species)
    if kind == "Moller":
        tb = pt.probTable(type="Moller", shell=mat.params["name_val"], func=ef.moller_dCS,
                          E_range=(Emin, E0), tol_E=tol, tol_W=tol, mat=mat,
                          mapTarget="../tables/integration", chunk_size=100, Wc=Wc)
    else:
        sh = mat.params["name_s"][::-1][0]
        tb = pt.probTable(type="Gryzinski", shell=sh, func=ef.gryz_dCS,
                          E_range=(Emin, E0), tol_E=tol, tol_W=tol, mat=mat,
                          mapTarget="../tables/integration", chunk_size=100)
    tb.set_Ws()
    tb.set_Es()
    tb.table = tb.computeBlock(tb.Es)
    tb.mapToMemory()
    tb.readFromMemory()
    return tb, mat


def part_tables():
    out = {"names": []}
    for cfg in [CFG1, CFG3] + CFG4:
        name, spc, E0, Emin, Wc, tol = cfg
        for kind in ("Moller", "Gryz"):
            t0 = time.time()
            tb, mat = build_table(kind, spc, E0, Emin, Wc, tol)
            key = "%s/%s" % (name, kind)
            cdf32 = np.asarray(tb.table.filled(0), dtype=np.float32)
            nE = cdf32.shape[0]
            rows = np.unique(np.linspace(0, nE - 1, min(nE, 48)).astype(np.int64))
            out["names"].append(key)
            out[key + "/spec"] = np.array([E0, Emin, Wc, tol])
            out[key + "/species"] = np.array(spc)
            out[key + "/Ws"] = np.asarray(tb.Ws, dtype=np.float32)
            out[key + "/Es"] = np.asarray(tb.Es, dtype=np.float32)
            out[key + "/rows"] = rows
            out[key + "/cdf_rows"] = cdf32[rows]
            out[key + "/nvalid"] = (cdf32 != 0).sum(axis=1).astype(np.int32)
            out[key + "/rowsum"] = cdf32.astype(np.float64).sum(axis=1)
            print(key, cdf32.shape, "%.1fs" % (time.time() - t0), flush=True)
    out["names"] = np.array(out["names"])
    np.savez_compressed(os.path.join(HERE, "tables.npz"), **out)


# ---------------------------------------------------------------------------
def _promote(tb):
    """Hold the float32 grids/table as float64 arrays (NumPy 1.x dtype flow)."""
    tb.Ws = np.asarray(tb.Ws, dtype=np.float64)
    tb.Es = np.asarray(tb.Es, dtype=np.float64)
    tb.table = ma.masked_array(np.asarray(tb.table.data, dtype=np.float64), tb.table.mask)
    return tb


def ds_tables(cfg):
    _, spc, E0, Emin, Wc, tol = cfg
    tm, mat = build_table("Moller", spc, E0, Emin, Wc, tol)
    tg, _ = build_table("Gryz", spc, E0, Emin, Wc, tol)
    return {"Moller": _promote(tm), "Gryz": [_promote(tg)]}, mat


SCAT_COLS = ["type", "E", "E_loss", "pol_angle", "az_angle", "pathl", "position", "energy"]
EL_COLS = ["outcome", "final_E", "final_dir", "last_pos"]


def run_ref_ds(mat, tables, E0, Emin, tilt, Wc, seed, maxz=INF_Z, scat_cols=SCAT_COLS, elastic="Ruth_vanilla",
               diffMFP=False):
    """One reference DS trajectory.  With diffMFP the discrete scatter class
    gets the extinction distance as a class attribute: its constructor reads
    self.xip_g, whose assignment is commented out (MC/tools/scattering.py:458),
    so without it the reference cannot run that path at all."""
    m = _load()
    sd = m["scattering"].scatter_discrete
    if diffMFP:
        sd.xip_g = mat.params["xip_g"]
    elif hasattr(sd, "xip_g"):
        del sd.xip_g
    d0 = np.array([-np.sin(np.radians(tilt)), 0.0, np.cos(np.radians(tilt))])
    el = m["electron"].electron(E0, Emin, np.array([0.0, 0.0, 0.0]), d0,
                                {"el_output": EL_COLS, "scat_output": scat_cols})
    random.seed(seed)
    m["singleScatter"].trajectory_DS(el, mat, Wc, BIG_MAXSCATT, maxz, elastic, tables, diffMFP)
    return el.el_output.dict, el.scat_output.dict


def run_ref_cont(mat, E0, Emin, tilt, seed, maxz=INF_Z, elastic="Ruth_vanilla"):
    """The loop of trajectory_cont_cl (MC/tools/singleScatter.py:205-239) with
    maxz passed, on the reference's classical scatter class and electron."""
    m = _load()
    d0 = np.array([-np.sin(np.radians(tilt)), 0.0, np.cos(np.radians(tilt))])
    el = m["electron"].electron(E0, Emin, np.array([0.0, 0.0, 0.0]), d0,
                                {"el_output": EL_COLS,
                                 "scat_output": ["type", "E_loss", "pol_angle", "az_angle", "pathl", "energy"]})
    random.seed(seed)
    while (el.outcome != "abs") and (el.outcome != "bks") and (el.outcome != "trsm"):
        sc = m["scattering"].scatter_continuous_classical(el, mat, elastic, None)
        sc.compute_pathl()
        el.update_xyz(sc.pathl, maxz)
        sc.compute_Eloss()
        el.update_energy(sc.E_loss)
        sc.compute_sAngles()
        el.update_direction(sc.c2_halfTheta, sc.halfPhi)
    return el.el_output.dict, el.scat_output.dict


def _flatten(el_list, sc_list, types):
    """Pack per-electron dicts into flat arrays with offsets."""
    out = {}
    ev_off, row_off = [0], [0]
    cols = {}
    rows = {"outcome": [], "final_E": [], "dx": [], "dy": [], "dz": [],
            "last_x": [], "last_y": [], "last_z": []}
    for eld, scd in zip(el_list, sc_list):
        n = len(scd["pathl"])
        ev_off.append(ev_off[-1] + n)
        for k, v in scd.items():
            if k == "position":
                for kk in ("x", "y", "z"):
                    cols.setdefault(kk, []).extend(float(a) for a in v[kk][:n])
            elif k == "type":
                cols.setdefault("type", []).extend(types.index(t) for t in v)
            else:
                cols.setdefault(k, []).extend(float(a) for a in v)
        nr = len(eld["outcome"])
        row_off.append(row_off[-1] + nr)
        rows["outcome"].extend(eld["outcome"])
        rows["final_E"].extend(float(a) for a in eld["final_E"])
        for kk in ("dx", "dy", "dz"):
            rows[kk].extend(float(a) for a in eld["final_dir"][kk])
        for kk in ("last_x", "last_y", "last_z"):
            rows[kk].extend(float(a) for a in eld["last_pos"][kk])
    for k, v in cols.items():
        out["ev/" + k] = np.asarray(v, dtype=np.int32 if k == "type" else np.float64)
    for k, v in rows.items():
        out["row/" + k] = np.asarray(v) if k == "outcome" else np.asarray(v, dtype=np.float64)
    out["ev_off"] = np.asarray(ev_off, dtype=np.int64)
    out["row_off"] = np.asarray(row_off, dtype=np.int64)
    return out


def type_labels(mat_params):
    return ["Ruth", "Moller", "Quinn"] + ["Gryz" + s for s in mat_params["name_s"]] + ["diff"]


def part_replay():
    out = {}
    # DS: cfg1 physics (Si 10 keV) and cfg3 physics (Au 30 keV, tilt 70); the
    # Nigram elastic cross sections; the diffraction channel in a Si film
    # (elastic model, diffMFP, thickness in A)
    for tag, cfg, tilt, n, base, elastic, diff, maxz in (
            ("ds_si", CFG1, 0.0, 24, 1000, "Ruth_vanilla", False, INF_Z),
            ("ds_au", CFG3, 70.0, 3, 2000, "Ruth_vanilla", False, INF_Z),
            ("ds_si_nigram", CFG1, 0.0, 8, 5000, "Ruth_nigram", False, INF_Z),
            ("ds_si_nigram_wdefl", CFG1, 0.0, 8, 6000, "Ruth_nigram_wDefl", False, INF_Z),
            ("ds_si_diff", CFG1, 0.0, 24, 7000, "Ruth_vanilla", True, 3000.0)):
        tables, mat = ds_tables(cfg)
        _, spc, E0, Emin, Wc, tol = cfg
        types = type_labels(mat.params)
        els, scs = [], []
        for k in range(n):
            with np.errstate(invalid="ignore"):
                e, s = run_ref_ds(mat, tables, E0, Emin, tilt, Wc, base + k, maxz=maxz, elastic=elastic,
                                  diffMFP=diff)
            els.append(e)
            scs.append(s)
        flat = _flatten(els, scs, types)
        for k, v in flat.items():
            out[tag + "/" + k] = v
        out[tag + "/elastic"] = np.array(elastic)
        out[tag + "/diffMFP"] = np.array(diff)
        out[tag + "/thickness"] = np.array(maxz)
        out[tag + "/cfg"] = np.array([E0, Emin, tilt, Wc, tol])
        out[tag + "/species"] = np.array(spc)
        out[tag + "/seeds"] = np.arange(base, base + n)
        print(tag, "events", flat["ev_off"][-1], "rows", flat["row_off"][-1], flush=True)
    # continuous, classical Bethe: Al 15 keV tilt 70 (cfg5 physics), Cu 20 keV tilt 70
    m = _load()
    for tag, spc, E0, tilt, n, base, elastic in (("cont_al", "Al", 15000.0, 70.0, 8, 3000, "Ruth_vanilla"),
                                                 ("cont_cu", "Cu", 20000.0, 70.0, 4, 4000, "Ruth_vanilla"),
                                                 ("cont_al_nigram", "Al", 15000.0, 70.0, 4, 8000, "Ruth_nigram")):
        mat = m["material"].material(spc)
        els, scs = [], []
        for k in range(n):
            e, s = run_ref_cont(mat, E0, 1000.0, tilt, base + k, elastic=elastic)
            els.append(e)
            scs.append(s)
        flat = _flatten(els, scs, [elastic])
        for k, v in flat.items():
            out[tag + "/" + k] = v
        out[tag + "/elastic"] = np.array(elastic)
        out[tag + "/cfg"] = np.array([E0, 1000.0, tilt])
        out[tag + "/species"] = np.array(spc)
        out[tag + "/seeds"] = np.arange(base, base + n)
        print(tag, "events", flat["ev_off"][-1], flush=True)
    np.savez_compressed(os.path.join(HERE, "replay.npz"), **out)


# ---------------------------------------------------------------------------
_STATS_CTX = {}


def _stats_job(args):
    job, n, base = args
    c = _STATS_CTX
    cols = ["type", "E", "E_loss", "pol_angle", "az_angle", "pathl", "position"]
    res = []
    for k in range(n):
        with np.errstate(invalid="ignore"):
            e, s = run_ref_ds(c["mat"], c["tables"], c["E0"], c["Emin"], c["tilt"], c["Wc"],
                              base + job * n + k, scat_cols=cols)
        types = [c["types"].index(t) for t in s["type"]]
        z = np.asarray(s["position"]["z"], dtype=np.float64)
        zmax = max(float(z.max()) if z.size else 0.0, float(e["last_pos"]["last_z"][0]))
        res.append(dict(
            outcome=e["outcome"][0], nrows=len(e["outcome"]),
            final_E=float(e["final_E"][0]),
            d=[float(e["final_dir"][kk][0]) for kk in ("dx", "dy", "dz")],
            p=[float(e["last_pos"][kk][0]) for kk in ("last_x", "last_y", "last_z")],
            nsteps=len(s["pathl"]), zmax=zmax,
            first=(types[0], float(s["pol_angle"][0]), float(s["E_loss"][0])),
            counts=np.bincount(types, minlength=len(c["types"])),
            nan=int(np.isnan(np.asarray(s["pol_angle"], dtype=np.float64)).sum()),
            # a thinned sample of all events: every 128th
            sample=np.column_stack([np.asarray(types)[::128],
                                    np.asarray(s["E"], dtype=np.float64)[::128],
                                    np.asarray(s["E_loss"], dtype=np.float64)[::128],
                                    np.asarray(s["pol_angle"], dtype=np.float64)[::128],
                                    np.asarray(s["az_angle"], dtype=np.float64)[::128]]),
        ))
    return res


STATS = [
    # tag, table cfg, tilt, electrons, electrons per job, seed base
    ("si10", CFG1, 0.0, 30000, 25, 1100000),
    ("au30", CFG3, 70.0, 3000, 5, 1200000),
    ("cu20t45", ("cfg4_Cu_20", "Cu", 20000.0, 1000.0, 100.0, 1e-3), 45.0, 12000, 10, 1300000),
    ("al5", ("cfg4_Al_5", "Al", 5000.0, 1000.0, 100.0, 1e-3), 0.0, 12000, 25, 1400000),
]


def part_stats(only=None):
    out = {}
    for tag, cfg, tilt, n_el, per_job, base in STATS:
        if only and tag not in only:
            continue
        t0 = time.time()
        tables, mat = ds_tables(cfg)
        _STATS_CTX.clear()
        _STATS_CTX.update(mat=mat, tables=tables, E0=cfg[2], Emin=cfg[3], Wc=cfg[4], tilt=tilt,
                          types=type_labels(mat.params))
        jobs = [(j, per_job, base) for j in range(n_el // per_job)]
        with mp.get_context("fork").Pool(os.cpu_count()) as pool:
            res = [r for chunk in pool.map(_stats_job, jobs, chunksize=1) for r in chunk]
        oc = {"bks": 1, "abs": 2, "trsm": 3, "trdf": 4, "long": 5}
        out[tag + "/cfg"] = np.array([cfg[2], cfg[3], tilt, cfg[4], cfg[5]])
        out[tag + "/species"] = np.array(cfg[1])
        out[tag + "/outcome"] = np.array([oc[r["outcome"]] for r in res], dtype=np.int8)
        out[tag + "/nrows"] = np.array([r["nrows"] for r in res], dtype=np.int8)
        out[tag + "/final_E"] = np.array([r["final_E"] for r in res], dtype=np.float32)
        out[tag + "/dir"] = np.array([r["d"] for r in res], dtype=np.float32)
        out[tag + "/last_pos"] = np.array([r["p"] for r in res], dtype=np.float32)
        out[tag + "/nsteps"] = np.array([r["nsteps"] for r in res], dtype=np.int32)
        out[tag + "/zmax"] = np.array([r["zmax"] for r in res], dtype=np.float32)
        out[tag + "/first"] = np.array([r["first"] for r in res], dtype=np.float32)
        out[tag + "/counts"] = np.sum([r["counts"] for r in res], axis=0)
        out[tag + "/nan"] = np.array(sum(r["nan"] for r in res))
        out[tag + "/sample"] = np.concatenate([r["sample"] for r in res]).astype(np.float32)
        dt = time.time() - t0
        out[tag + "/wall_s"] = np.array([dt, os.cpu_count()])
        eta = float(np.mean(out[tag + "/outcome"] == 1))
        print("%s: N=%d eta=%.4f steps/el=%.1f %.1fs on %d procs" % (
            tag, len(res), eta, out[tag + "/nsteps"].mean(), dt, os.cpu_count()), flush=True)
    path = os.path.join(HERE, "ref_stats.npz")
    if only and os.path.exists(path):
        old = dict(np.load(path))
        old.update(out)
        out = old
    np.savez_compressed(path, **out)


if __name__ == "__main__":
    parts = sys.argv[1:] or ["physics", "tables", "replay"]
    _load()
    for p in parts:
        if p == "physics":
            part_physics()
        elif p == "tables":
            part_tables()
        elif p == "replay":
            part_replay()
        elif p.startswith("stats"):
            only = p.split(":")[1].split(",") if ":" in p else None
            part_stats(only)
        else:
            raise SystemExit("unknown part " + p)
