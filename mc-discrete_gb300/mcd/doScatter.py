"""Whole-simulation driver: the GPU counterpart of MC/doScatter.py.

main() reads an input.file, transports num_el electrons on the GPU in
chunks and writes the reference's three tables under the reference's file
name (MC/doScatter.py:175-186):

  input   the parameters as strings (MC/doScatter.py:197-200)
  els     electron_output columns, one row per outcome row of an electron
          (a 'bks' followed by 'abs' in the same step gives two rows)
  scats   scatter_output columns, one row per event, electrons in order

with the column splitting of MC/tools/fileTools.py:67-99 (final_dir ->
dx, dy, dz; position -> x, y, z; last_pos -> last_x, last_y, last_z).
The tables are written to an HDF5 store through pandas when pandas and
PyTables are importable, as the reference does (string columns sized to
their longest value rather than the reference's 6 characters, which cut
shell labels such as 'Gryz3s3p3d'); otherwise to a NumPy .npz file with
keys 'input/<name>', 'els/<column>' and 'scats/<column>'.

The pool of CPU workers (MapScatterer, MC/doScatter.py:22-95) has no
counterpart: each chunk is one launch of the persistent batched kernel
(with an event ring when scatter_output is asked for), or a plain launch
when a block size is given.
"""
import argparse
import json
import math
import os
import time

import numpy as np

from . import _lib
from .config import readInput, with_defaults
from .engine import Batch, collect, launch, make_sim, mode_of, RunBuffers, RunResult, use_sigma_table
from .tables import ds_tables

EL_COLS = ("outcome", "final_E", "final_dir", "last_pos")
SCAT_COLS = ("type", "E", "E_loss", "pol_angle", "az_angle", "pathl", "position", "energy")


def store_name(inputPar, path="../data/", ext=".h5"):
    """MC/doScatter.py:175-186."""
    p = inputPar
    return (path + "TRSM_diff:" + str(p["diffMFP"]) + "_thick:" + str(p["thickness"]) + "_mat:" +
            str(p["material"]) + "_mode:" + str(p["mode"]) + "_elastic:" + str(p["elastic"]) + "_tilt:" +
            str(p["s_tilt"]) + "_Emin:" + str(p["Emin"]) + "_E0:" + str(p["E0"]) + "_tolE:" + str(p["tol_E"]) +
            "_tolW:" + str(p["tol_W"]) + ext)


def type_labels(mat, mode, elastic):
    """Channel code -> the reference's 'type' label (scattering.py:483-516,
    :834 for continuous mode, where the label is the elastic model name)."""
    if mode == _lib.MODE_CONT:
        return np.array([elastic] * _lib.CH_DIFF + [elastic])
    names = ["Ruth", "Moller", "Quinn"] + ["Gryz" + mat.shell_name[k].value.decode() for k in range(mat.n_shells)]
    names += [""] * (_lib.CH_DIFF - len(names)) + ["diff"]
    return np.array(names)


# scatter_output column -> ring record fields it needs ('type' is in the header)
COL_FIELDS = {"type": 0, "E": _lib.EV_E, "E_loss": _lib.EV_W, "pol_angle": _lib.EV_C2, "az_angle": _lib.EV_PHI,
              "pathl": _lib.EV_PATHL, "position": _lib.EV_POS, "energy": _lib.EV_E | _lib.EV_W}


def ring_fields(sc_cols):
    """The ring field mask that carries exactly the requested columns."""
    f = 0
    for c in sc_cols:
        f |= COL_FIELDS.get(c, 0)
    return f if f else _lib.EV_PATHL     # 'type' alone: the smallest record with a field


def chunk_tables(res, n, el_cols, sc_cols, labels):
    """Column arrays of one chunk of n electrons from its device rows."""
    e = res.electrons
    two = (e["flags"] & 1).astype(bool)          # a second ('abs') row
    reps = 1 + two.astype(np.int64)
    els = {}
    if "outcome" in el_cols:
        oc = np.array(_lib.OUTCOME_NAMES)[e["outcome"].astype(np.int64)]
        oc = np.repeat(oc, reps)
        second = np.cumsum(reps) - 1
        oc[second[two]] = "abs"
        els["outcome"] = oc
    if "final_E" in el_cols:
        els["final_E"] = np.repeat(e["final_E"].astype(np.float64), reps)
    if "final_dir" in el_cols:
        for j, k in enumerate(("dx", "dy", "dz")):
            els[k] = np.repeat(e["dir"][:, j].astype(np.float64), reps)
    if "last_pos" in el_cols:
        for j, k in enumerate(("last_x", "last_y", "last_z")):
            els[k] = np.repeat(e["last_pos"][:, j].astype(np.float64), reps)
    scats = {}
    if sc_cols:
        ev = res.events
        ev = ev[np.lexsort((ev["step_chan"] >> 5, ev["electron"]))]
        ch = (ev["step_chan"] & 31).astype(np.int64)
        for c in sc_cols:
            if c == "type":
                scats["type"] = labels[ch]
            elif c == "E":
                scats["E"] = ev["E"].astype(np.float64)
            elif c == "E_loss":
                scats["E_loss"] = ev["W"].astype(np.float64)
            elif c == "pol_angle":
                scats["pol_angle"] = ev["c2"].astype(np.float64)
            elif c == "az_angle":
                scats["az_angle"] = ev["half_phi"].astype(np.float64)
            elif c == "pathl":
                scats["pathl"] = ev["pathl"].astype(np.float64)
            elif c == "position":
                for k in ("x", "y", "z"):
                    scats[k] = ev[k].astype(np.float64)
            elif c == "energy":
                scats["energy"] = ev["E"].astype(np.float64) - ev["W"].astype(np.float64)
    return els, scats


class NpzWriter:
    """Collects the tables and writes one .npz file at close()."""

    def __init__(self, name, inputPar):
        self.name = name
        self.parts = {"els": {}, "scats": {}}
        self.input = {k: str(v) for k, v in inputPar.items()}

    def append(self, key, cols):
        for c, v in cols.items():
            self.parts[key].setdefault(c, []).append(v)

    def close(self):
        out = {"input/" + k: np.array(v) for k, v in self.input.items()}
        for key, cols in self.parts.items():
            for c, chunks in cols.items():
                out[key + "/" + c] = np.concatenate(chunks)
        np.savez(self.name, **out)


class HdfWriter:
    """The reference's store layout through pandas.HDFStore: 'input' as the
    one-row frame of the parameters (MC/doScatter.py:62-67), 'els' and
    'scats' appended in tables format with data columns
    (MC/doScatter.py:112-117).  String columns get room for the longest
    label (the reference's 6 characters cut 'Gryz3s3p3d'), fixed when the
    first chunk creates the table."""

    def __init__(self, name, inputPar):
        import pandas as pd
        self.pd = pd
        self.name = name
        self.store = pd.HDFStore(name, mode="w")
        self.store["input"] = pd.DataFrame(pd.Series(inputPar)).T
        self.width = {"els": {"outcome": 6}, "scats": {"type": 24}}

    def append(self, key, cols):
        if not cols:
            return
        df = self.pd.DataFrame(cols)
        sizes = {c: max(w, int(df[c].str.len().max() or 0)) for c, w in self.width[key].items() if c in df}
        self.store.put(key, df, format="table", data_columns=True, append=True, min_itemsize=sizes)

    def close(self):
        self.store.close()


def _hdf_available():
    try:
        import pandas  # noqa: F401
        import tables  # noqa: F401
        return True
    except ImportError:
        return False


def run(inputPar, path="../data/", fmt=None, chunk=100_000, seed=0, events_per_electron=1000, block_size=0):
    """Transport inputPar['num_el'] electrons and write the tables, and a JSON
    run record beside them (parameters, seed, outcome and channel counts,
    eta and its standard error, events/s, the OR of the status words).
    fmt: 'h5', 'npz' or None (h5 when pandas and PyTables are present).
    Returns the file name."""
    p = with_defaults(inputPar)
    fmt = fmt or ("h5" if _hdf_available() else "npz")
    name = store_name(p, path, ".h5" if fmt == "h5" else ".npz")
    os.makedirs(path or ".", exist_ok=True)
    if os.path.exists(name):
        os.remove(name)
    writer = HdfWriter(name, p) if fmt == "h5" else NpzWriter(name, p)
    el_cols = [c for c in p.get("electron_output", []) if c]
    sc_cols = [c for c in p.get("scatter_output", []) if c]
    for c in el_cols:
        if c not in EL_COLS:
            raise ValueError("electron_output column %r is not produced (have %s)" % (c, EL_COLS))
    for c in sc_cols:
        if c not in SCAT_COLS:
            raise ValueError("scatter_output column %r is not produced (have %s)" % (c, SCAT_COLS))
    mode = mode_of(p)
    mat = _lib.material(p["material"])
    labels = type_labels(mat, mode, p.get("elastic", "Ruth_vanilla"))
    tables = (ds_tables(mat, p["E0"], p["Emin"], p["Wc"], p["tol_E"], p["tol_W"])
              if mode == _lib.MODE_DS else None)
    total = int(p["num_el"])
    epe = float(events_per_electron)
    first = 0
    record = {"outcomes": {k: 0 for k in _lib.OUTCOME_NAMES}, "channels": {}, "events": 0, "double_rows": 0,
              "nan_events": 0, "status": 0, "gpu_s": 0.0, "launches": 0}
    t_start = time.perf_counter()
    while first < total:
        n = min(int(chunk), total - first)
        if block_size:
            res = _plain_chunk(p, n, seed, first, mat, tables, block_size, sc_cols, epe, record)
        else:
            res = _batched_chunk(p, n, seed, first, sc_cols, epe, record)
        if sc_cols:
            epe = max(epe, res.events_total / n)
        _add_to_record(record, res, labels)
        els, scats = chunk_tables(res, n, el_cols, sc_cols, labels)
        writer.append("els", els)
        writer.append("scats", scats)
        first += n
    writer.close()
    _write_record(name, p, seed, total, record, time.perf_counter() - t_start)
    return name


def _plain_chunk(p, n, seed, first, mat, tables, block_size, sc_cols, epe, record):
    """One chunk as one plain launch, with its events in a device ring."""
    sim = make_sim(p, n, seed, first, tally_flags=_lib.TALLY_CHANNELS)
    use_sigma_table(sim, mat)
    cap = int(1.3 * epe * n) + 4096 if sc_cols else 0
    while True:
        bufs = RunBuffers(n, _lib.FP32, True, cap, ring_fields=ring_fields(sc_cols))
        bufs.zero()
        t0 = time.perf_counter()
        launch(sim, mat, tables, bufs, block_size)
        res = collect(bufs)
        record["gpu_s"] += time.perf_counter() - t0
        record["launches"] += 1
        if not sc_cols or res.events_total <= cap:
            return res
        cap = int(1.2 * res.events_total) + 4096     # same counters: the re-run is exact


def _batched_chunk(p, n, seed, first, sc_cols, epe, record):
    """One chunk on the persistent kernel (a warp refills its lanes from the
    queue as electrons finish), keeping the per-electron rows and, for
    scatter_output, every event in a device ring; the same electrons and
    cross-section table as a plain launch, so the same rows and events."""
    from .autotune import tune
    b = Batch([dict(p, num_el=n)], seed=seed, first_electron=first, electrons=True, tally_channels=True)
    t_ = tune(b)[0]
    cap = int(1.3 * epe * n) + 4096
    while True:
        t0 = time.perf_counter()
        if sc_cols:
            tallies, status, events, total = b.run_events(cap, ring_fields(sc_cols), t_)
        else:
            (tallies, status), events, total = b.run(t_), None, 0
        rows = b.electrons(0)
        record["gpu_s"] += time.perf_counter() - t0
        record["launches"] += 1
        if not sc_cols or total <= cap:
            return RunResult(tallies[0], status, rows, events, total)
        cap = int(1.2 * total) + 4096     # same counters: the re-run is exact


def _add_to_record(record, res, labels):
    t = res.tally
    for k in _lib.OUTCOME_NAMES:
        record["outcomes"][k] += int(t[k])
    for code, count in enumerate(t["channel"]):
        if count:
            lab = str(labels[code]) if code < len(labels) and labels[code] else str(code)
            record["channels"][lab] = record["channels"].get(lab, 0) + int(count)
    for k in ("events", "double_rows", "nan_events"):
        record[k] += int(t[k])
    record["status"] |= int(res.status)


def _device_name():
    import torch
    return torch.cuda.get_device_name(torch.cuda.current_device())


def _write_record(name, p, seed, n, record, wall_s):
    """The run record: <store name>.json."""
    bks = record["outcomes"]["bks"]
    eta = bks / n if n else float("nan")
    rec = {"file": os.path.basename(name), "input": {k: str(v) for k, v in p.items()}, "seed": int(seed),
           "num_el": n, **record, "eta": eta, "eta_sigma": math.sqrt(eta * (1.0 - eta) / n) if n else float("nan"),
           "events_per_s": record["events"] / record["gpu_s"] if record["gpu_s"] > 0 else None,
           "wall_s": wall_s, "device": _device_name()}
    with open(os.path.splitext(name)[0] + ".json", "w") as f:
        json.dump(rec, f, indent=1)


def main(argv=None):
    """`python -m mcd -i input.file`, as `python doScatter.py -i input.file`."""
    ap = argparse.ArgumentParser(prog="python -m mcd", description=__doc__.splitlines()[0])
    ap.add_argument("-i", "--ifile", default="../inputFile/input.file", help="input file")
    ap.add_argument("-o", "--out", default="../data/", help="output directory")
    ap.add_argument("--format", choices=("h5", "npz"), default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--chunk", type=int, default=100_000, help="electrons per kernel launch")
    ap.add_argument("--block-size", type=int, default=0,
                    help="threads per block (8, 16 or a multiple of 32 up to 256; 0 = automatic)")
    a = ap.parse_args(argv)
    p = readInput(a.ifile)
    print(" - Number of incident electrons: %s" % p["num_el"])
    print(" - Material is: %s" % p["material"])
    print(" - Scattering mode is: %s" % p["mode"])
    print(" - Elastic scattering mode is: %s" % p.get("elastic", "Ruth_vanilla"))
    out = a.out if a.out.endswith("/") else a.out + "/"
    name = run(p, out, a.format, a.chunk, a.seed, block_size=a.block_size)
    print(" BSE data had been written to ", name)
    return name
