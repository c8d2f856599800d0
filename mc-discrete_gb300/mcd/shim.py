"""Drop-in replacements for the reference's trajectory workers.

    multiTraj_DS(inputPar, numTraj, material, tables, thingsToSave)
        (MC/tools/multiScatter.py:66-116)
    multiTraj_cont(inputPar, numTraj, material, thingsToSave, tables)
        (MC/tools/multiScatter.py:171-229)

Both return a list with one {'els': dict, 'scats': dict} per electron, with
the reference's column names (MC/tools/fileTools.py:193-242): 'final_dir'
expands to dx/dy/dz, 'position' to x/y/z, 'last_pos' to last_x/last_y/last_z.
An electron that leaves through the surface and falls below Emin in the same
step gets the reference's second 'abs' row (MC/tools/electron.py:52-54).

The work runs on the GPU.  `material` and `tables` keep the reference's
signatures and are not used: the material comes from inputPar['material']
and the tables are built on the GPU once per parameter set.  Each call
takes a fresh range of Philox electron indices, so repeated calls give new
trajectories; pass `seed` in inputPar to choose the stream.
"""
import itertools
import threading

import numpy as np

from . import _lib
from .config import with_defaults
from .doScatter import EL_COLS, SCAT_COLS, ring_fields, type_labels
from .engine import collect, launch, make_sim, mode_of, RunBuffers, use_sigma_table
from .tables import ds_tables

_counter = itertools.count()
_lock = threading.Lock()


def _next_range(n):
    with _lock:
        k = next(_counter)
    return k * (1 << 32), n


def _assemble(res, n, wanted, mat, mode, elastic):
    el_cols = list(wanted.get("el_output", []))
    sc_cols = list(wanted.get("scat_output", []))
    for c in el_cols:
        if c not in EL_COLS:
            raise ValueError("electron_output column %r is not produced (have %s)" % (c, EL_COLS))
    for c in sc_cols:
        if c not in SCAT_COLS:
            raise ValueError("scatter_output column %r is not produced (have %s)" % (c, SCAT_COLS))
    e = res.electrons
    names = type_labels(mat, mode, elastic)
    ev = res.events
    order = np.lexsort((ev["step_chan"] >> 5, ev["electron"])) if ev is not None and ev.size else None
    if order is not None:
        ev = ev[order]
        starts = np.searchsorted(ev["electron"], np.arange(n + 1))
    out = []
    for i in range(n):
        oc = _lib.OUTCOME_NAMES[int(e["outcome"][i])]
        rows = [oc]
        if e["flags"][i] & 1:
            rows.append("abs")
        els = {}
        for c in el_cols:
            if c == "outcome":
                els["outcome"] = rows
            elif c == "final_E":
                els["final_E"] = [float(e["final_E"][i])] * len(rows)
            elif c == "final_dir":
                d = e["dir"][i]
                els["final_dir"] = {k: [float(d[j])] * len(rows) for j, k in enumerate(("dx", "dy", "dz"))}
            elif c == "last_pos":
                p = e["last_pos"][i]
                els["last_pos"] = {k: [float(p[j])] * len(rows)
                                   for j, k in enumerate(("last_x", "last_y", "last_z"))}
        scats = {}
        if sc_cols:
            seg = ev[starts[i]:starts[i + 1]] if order is not None else ev[:0]
            ch = (seg["step_chan"] & 31).astype(int)
            for c in sc_cols:
                if c == "type":
                    scats["type"] = names[ch].tolist()
                elif c == "E":
                    scats["E"] = seg["E"].astype(float).tolist()
                elif c == "E_loss":
                    scats["E_loss"] = seg["W"].astype(float).tolist()
                elif c == "pol_angle":
                    scats["pol_angle"] = seg["c2"].astype(float).tolist()
                elif c == "az_angle":
                    scats["az_angle"] = seg["half_phi"].astype(float).tolist()
                elif c == "pathl":
                    scats["pathl"] = seg["pathl"].astype(float).tolist()
                elif c == "position":
                    scats["position"] = {k: seg[k].astype(float).tolist() for k in ("x", "y", "z")}
                elif c == "energy":
                    scats["energy"] = (seg["E"].astype(float) - seg["W"].astype(float)).tolist()
        out.append({"els": els, "scats": scats})
    return out


def _run_traj(inputPar, numTraj, thingsToSave):
    p = with_defaults(inputPar)
    mode = mode_of(p)
    mat = _lib.material(p["material"])
    first, n = _next_range(int(numTraj))
    seed = int(p.get("seed", 0))
    sim = make_sim(p, n, seed, first)
    use_sigma_table(sim, mat)
    tables = (ds_tables(mat, p["E0"], p["Emin"], p["Wc"], p["tol_E"], p["tol_W"])
              if mode == _lib.MODE_DS else None)
    want_events = bool(thingsToSave.get("scat_output"))
    cap = n * 2048 if want_events else 0
    # the ring records carry only the requested scatter_output columns
    fields = ring_fields(list(thingsToSave.get("scat_output", [])))
    while True:
        bufs = RunBuffers(n, _lib.FP32, True, cap, ring_fields=fields)
        bufs.zero()
        launch(sim, mat, tables, bufs)
        res = collect(bufs)
        if not want_events or res.events_total <= cap:
            break
        cap = int(res.events_total * 1.25) + 1024   # the stream is counter-based: re-running is exact
    return _assemble(res, n, thingsToSave, mat, mode, p.get("elastic", "Ruth_vanilla"))


def multiTraj_DS(inputPar, numTraj, material=None, tables=None, thingsToSave=None):  # noqa: N802
    """numTraj DS trajectories (MC/tools/multiScatter.py:66)."""
    if thingsToSave is None:
        thingsToSave = {"el_output": list(EL_COLS), "scat_output": []}
    p = dict(inputPar)
    p["mode"] = "DS"
    return _run_traj(p, numTraj, thingsToSave)


def multiTraj_cont(inputPar, numTraj, material=None, thingsToSave=None, tables=None):  # noqa: N802
    """numTraj continuous-slowing-down trajectories (MC/tools/multiScatter.py:171)."""
    if thingsToSave is None:
        thingsToSave = {"el_output": list(EL_COLS), "scat_output": []}
    p = dict(inputPar)
    if "DS" in p.get("mode", "cont"):
        p["mode"] = "cont"
    return _run_traj(p, numTraj, thingsToSave)
