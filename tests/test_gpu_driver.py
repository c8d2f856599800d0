"""The whole-simulation driver on the GPU: `python -m mcd -i input.file`
writes the reference's input / els / scats tables (here as .npz; HDF5 where
pandas and PyTables exist), consistent with the run's own tallies, and a
JSON run record beside them."""
import subprocess
import sys

import numpy as np
import pytest

from mcd import _lib, config, doScatter, engine

pytestmark = pytest.mark.gpu

INPUT = """num_el   : 3000
E0       : 10000
Emin     : 1000
material : Si
s_tilt   : 0
mode     : DS
Wc       : 100
tol_E    : 1e-3
tol_W    : 1e-3
maxScatt : 100000
electron_output : outcome, final_E, final_dir, last_pos
scatter_output : type, E, E_loss, pol_angle, az_angle, pathl, position, energy
"""


def test_cli_writes_reference_tables(tmp_path):
    f = tmp_path / "input.file"
    f.write_text(INPUT)
    out = str(tmp_path / "data") + "/"
    root = __file__.rsplit("/tests/", 1)[0]
    r = subprocess.run([sys.executable, "-m", "mcd", "-i", str(f), "-o", out, "--format", "npz", "--chunk", "1000"],
                       cwd=root + "/mc-discrete_gb300", capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    p = config.readInput(str(f))
    name = doScatter.store_name(config.with_defaults(p), out, ".npz")
    z = np.load(name)
    assert str(z["input/material"]) == "Si" and str(z["input/num_el"]) == "3000"
    oc = z["els/outcome"]
    # the same electrons (indices 0..2999, seed 0) with the same cross-section
    # table, as plain launches: the same tallies and the same events
    g = engine.run(p, num_el=3000, seed=0, tabulated=True, ring_capacity=3000 * 1500)
    ev = g.events[np.lexsort((g.events["step_chan"] >> 5, g.events["electron"]))]
    assert np.array_equal(z["scats/E"], ev["E"].astype(np.float64))
    assert np.array_equal(z["scats/E_loss"], ev["W"].astype(np.float64))
    t = g.tally
    assert (oc == "bks").sum() == t["bks"] and (oc == "abs").sum() == t["abs"] + t["double_rows"]
    assert oc.size == 3000 + t["double_rows"]
    assert z["scats/type"].size == t["events"]
    for c in ("E", "E_loss", "pol_angle", "az_angle", "pathl", "x", "y", "z", "energy"):
        assert z["scats/" + c].size == t["events"], c
    assert set(np.unique(z["scats/type"])) <= {"Ruth", "Moller", "Quinn", "Gryz1s", "Gryz2s", "Gryz2p"}
    assert np.allclose(z["scats/energy"], z["scats/E"] - z["scats/E_loss"])
    for c in ("dx", "dy", "dz", "last_x", "last_y", "last_z", "final_E"):
        assert z["els/" + c].size == oc.size
    # the run record beside the tables
    import json
    rec = json.load(open(name[:-4] + ".json"))
    assert rec["num_el"] == 3000 and rec["seed"] == 0 and rec["launches"] == 3
    assert rec["outcomes"]["bks"] == t["bks"] and rec["events"] == t["events"]
    assert sum(rec["channels"].values()) == t["events"]
    assert set(rec["channels"]) <= {"Ruth", "Moller", "Quinn", "Gryz1s", "Gryz2s", "Gryz2p"}
    assert abs(rec["eta"] - t["bks"] / 3000) < 1e-12 and rec["events_per_s"] > 0
    assert rec["status"] & ~_lib.FLAG_NAN == 0          # the reference's NaN angles may be flagged


def test_rows_only_run_uses_the_batched_kernel_with_the_same_rows(tmp_path, monkeypatch):
    """Without scatter_output the driver runs each chunk on the persistent
    kernel; its rows equal those of plain launches of the same electrons."""
    monkeypatch.setenv("MCD_CACHE_DIR", str(tmp_path / "cache"))
    p = config.parse_input(INPUT.replace("scatter_output : type, E, E_loss, pol_angle, az_angle, pathl, position, energy",
                                         "scatter_output :"))
    assert not [c for c in p.get("scatter_output", []) if c]
    name = doScatter.run(p, str(tmp_path) + "/", "npz", chunk=1000, seed=0)
    z = np.load(name)
    g = engine.run(p, num_el=3000, seed=0, tabulated=True)
    e = g.electrons
    reps = 1 + (e["flags"] & 1).astype(np.int64)
    assert np.array_equal(z["els/final_E"], np.repeat(e["final_E"].astype(np.float64), reps))
    assert np.array_equal(z["els/dz"], np.repeat(e["dir"][:, 2].astype(np.float64), reps))
    assert "scats/type" not in z.files
