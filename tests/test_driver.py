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


class _Col:
    def __init__(self, v):
        self.v = np.asarray(v)

    @property
    def str(self):
        return self

    def len(self):
        return _Col([len(x) for x in self.v])

    def max(self):
        return self.v.max() if self.v.size else 0


class _Frame:
    def __init__(self, data=None):
        if isinstance(data, _Series):
            self.cols = {0: data}
        else:
            self.cols = {k: np.asarray(v) for k, v in dict(data).items()}
        self.transposed = False

    @property
    def T(self):
        f = _Frame({})
        f.cols = self.cols
        f.transposed = not self.transposed
        return f

    def __contains__(self, c):
        return c in self.cols

    def __getitem__(self, c):
        return _Col(self.cols[c])


class _Series:
    def __init__(self, d):
        self.d = dict(d)


class _Store:
    def __init__(self, name, mode="a"):
        self.name, self.mode = name, mode
        self.items, self.puts, self.closed = {}, [], False

    def __setitem__(self, k, v):
        self.items[k] = v

    def put(self, key, df, **kw):
        self.puts.append((key, df, kw))

    def close(self):
        self.closed = True


def test_hdf_writer_drives_pandas_like_the_reference(monkeypatch):
    """The HDF5 branch (pandas and PyTables are absent here) against a
    recording stand-in of the pandas calls the reference makes: the one-row
    input frame (MC/doScatter.py:62-67) and tables-format appends with data
    columns and string sizes (MC/doScatter.py:112-117)."""
    import types
    fake = types.ModuleType("pandas")
    fake.HDFStore, fake.DataFrame, fake.Series = _Store, _Frame, _Series
    monkeypatch.setitem(__import__("sys").modules, "pandas", fake)
    p = config.with_defaults(dict(material="Au", mode="DS", E0=20000.0, Emin=1000.0, s_tilt=0.0,
                                  tol_E=1e-3, tol_W=1e-3, electron_output=["outcome"], scatter_output=["type"]))
    w = doScatter.HdfWriter("x.h5", p)
    assert w.store.mode == "w"
    inp = w.store.items["input"]
    assert inp.transposed and inp.cols[0].d == p
    w.append("els", {"outcome": np.array(["bks", "abs"]), "final_E": np.array([1.0, 2.0])})
    w.append("scats", {"type": np.array(["Ruth", "Gryz3s3p3d"]), "E": np.array([1.0, 2.0])})
    w.append("scats", {})
    w.close()
    assert w.store.closed
    assert [k for k, _, _ in w.store.puts] == ["els", "scats"]
    for key, df, kw in w.store.puts:
        assert kw["format"] == "table" and kw["data_columns"] is True and kw["append"] is True
    assert w.store.puts[0][2]["min_itemsize"] == {"outcome": 6}
    assert w.store.puts[1][2]["min_itemsize"] == {"type": 24}
    assert list(w.store.puts[1][1].cols["type"]) == ["Ruth", "Gryz3s3p3d"]
