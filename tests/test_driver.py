"""The whole-simulation driver's host logic (mcd.doScatter), without a GPU:
the reference's store name (MC/doScatter.py:175-186) and the assembly of
the els / scats tables from one chunk's device rows (second 'abs' rows,
the column splitting of MC/tools/fileTools.py:67-99, event order)."""
import numpy as np

from mcd import _lib, config, doScatter
from mcd.engine import EVENT_DTYPE


class Res:
    def __init__(self, electrons, events):
        self.electrons = electrons
        self.events = events


def test_store_name_matches_reference_pattern():
    p = config.with_defaults(dict(material="Si", mode="DS", E0=10000.0, Emin=1000.0, s_tilt=0.0,
                                  tol_E=1e-3, tol_W=1e-3))
    assert doScatter.store_name(p) == ("../data/TRSM_diff:False_thick:1e+30_mat:Si_mode:DS_elastic:Ruth_vanilla"
                                       "_tilt:0.0_Emin:1000.0_E0:10000.0_tolE:0.001_tolW:0.001.h5")


def test_chunk_tables():
    n = 3
    e = dict(outcome=np.array([1, 2, 1], np.uint8), flags=np.array([1, 0, 0], np.uint8),
             final_E=np.array([5000.0, 1500.0, 7000.0], np.float32),
             dir=np.arange(9, dtype=np.float32).reshape(3, 3), last_pos=-np.arange(9, dtype=np.float32).reshape(3, 3))
    ev = np.zeros(5, EVENT_DTYPE)
    # events arrive interleaved across electrons; the table lists them per electron, in order
    ev["electron"] = [2, 0, 0, 2, 1]
    ev["step_chan"] = [(0 << 5) | 0, (1 << 5) | 2, (0 << 5) | 1, (1 << 5) | 3, (0 << 5) | 11]
    ev["E"] = [10.0, 20.0, 30.0, 40.0, 50.0]
    ev["W"] = [1.0, 2.0, 3.0, 4.0, 5.0]
    ev["x"] = [0.5, 1.5, 2.5, 3.5, 4.5]
    mat = _lib.material("Si")
    labels = doScatter.type_labels(mat, _lib.MODE_DS, "Ruth_vanilla")
    els, scats = doScatter.chunk_tables(Res(e, ev), n, ["outcome", "final_E", "final_dir", "last_pos"],
                                        ["type", "E", "E_loss", "position", "energy"], labels)
    # electron 0 backscattered and then fell below Emin in the same step: two rows
    assert list(els["outcome"]) == ["bks", "abs", "abs", "bks"]
    assert list(els["final_E"]) == [5000.0, 5000.0, 1500.0, 7000.0]
    assert list(els["dx"]) == [0.0, 0.0, 3.0, 6.0] and list(els["last_z"]) == [-2.0, -2.0, -5.0, -8.0]
    assert list(scats["type"]) == ["Moller", "Quinn", "diff", "Ruth", "Gryz1s"]
    assert list(scats["E"]) == [30.0, 20.0, 50.0, 10.0, 40.0]
    assert list(scats["energy"]) == [27.0, 18.0, 45.0, 9.0, 36.0]
    assert set(scats) == {"type", "E", "E_loss", "x", "y", "z", "energy"}
    cont = doScatter.type_labels(mat, _lib.MODE_CONT, "Ruth_nigram")
    assert cont[_lib.CH_RUTH] == "Ruth_nigram"


def test_ring_fields_follow_requested_columns():
    assert doScatter.ring_fields(["type", "E_loss", "pol_angle", "pathl", "position"]) == (
        _lib.EV_W | _lib.EV_C2 | _lib.EV_PATHL | _lib.EV_POS)
    assert doScatter.ring_fields(["energy"]) == _lib.EV_E | _lib.EV_W
    assert doScatter.ring_fields(list(doScatter.SCAT_COLS)) == _lib.EV_ALL

