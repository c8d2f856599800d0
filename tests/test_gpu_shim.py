"""The reference-facing worker functions return the reference's columns."""
import numpy as np
import pytest

import mcd
from _gpu_util import input_par

pytestmark = pytest.mark.gpu

SAVE = {"el_output": ["outcome", "final_E", "final_dir", "last_pos"],
        "scat_output": ["type", "E", "E_loss", "pol_angle", "az_angle", "pathl", "position", "energy"]}


def test_multitraj_ds_columns():
    p = input_par("Si", 10000.0, 1000.0, 0.0)
    res = mcd.multiTraj_DS(p, 8, None, None, SAVE)
    assert len(res) == 8
    names = {"Ruth", "Moller", "Quinn", "Gryz1s", "Gryz2s", "Gryz2p"}
    for r in res:
        els, sc = r["els"], r["scats"]
        assert els["outcome"][0] in ("bks", "abs", "trsm", "long")
        assert len(els["outcome"]) in (1, 2)
        if len(els["outcome"]) == 2:
            assert els["outcome"] == ["bks", "abs"]
        assert set(els["final_dir"]) == {"dx", "dy", "dz"}
        assert set(els["last_pos"]) == {"last_x", "last_y", "last_z"}
        n = len(sc["type"])
        assert n > 0 and set(sc["type"]) <= names
        for k in ("E", "E_loss", "pol_angle", "az_angle", "pathl", "energy"):
            assert len(sc[k]) == n
        assert set(sc["position"]) == {"x", "y", "z"} and len(sc["position"]["z"]) == n
        E = np.array(sc["E"])
        assert E[0] == 10000.0 and np.all(np.diff(E) <= 0)
        assert np.allclose(np.array(sc["energy"]), E - np.array(sc["E_loss"]), rtol=1e-6)
        assert sc["position"]["z"][0] == 0.0
        assert np.all(np.array(sc["az_angle"]) < np.pi + 1e-6)


def test_multitraj_calls_give_new_electrons():
    p = input_par("Al", 5000.0, 1000.0, 0.0)
    a = mcd.multiTraj_DS(p, 4, None, None, {"el_output": ["final_E"], "scat_output": ["pathl"]})
    b = mcd.multiTraj_DS(p, 4, None, None, {"el_output": ["final_E"], "scat_output": ["pathl"]})
    assert [r["scats"]["pathl"][:3] for r in a] != [r["scats"]["pathl"][:3] for r in b]


def test_multitraj_cont_columns():
    p = input_par("Cu", 20000.0, 1000.0, 70.0, mode="cont", bethe="JL")
    save = {"el_output": ["outcome", "final_E"], "scat_output": ["type", "E_loss", "pathl", "energy"]}
    res = mcd.multiTraj_cont(p, 6, None, save, None)
    assert len(res) == 6
    for r in res:
        assert set(r["scats"]["type"]) == {"Ruth_vanilla"}
        assert r["els"]["outcome"][0] in ("bks", "abs", "trsm")


def test_unknown_column_is_rejected():
    p = input_par("Si", 10000.0, 1000.0, 0.0)
    with pytest.raises(ValueError):
        mcd.multiTraj_DS(p, 1, None, None, {"el_output": ["outcome"], "scat_output": ["direction"]})
