"""Edge cases of the transport entry points: empty simulations alone and
mixed into a batch, the largest batch (256 simulations), the event limit
('long' rows), a film thin enough that every electron is transmitted on
its first step, a beam barely above Emin, electron indices above 2^32
(the Philox counter's high word) and the plain kernel's block sizes, each
against the oracle or the plain kernel."""
import numpy as np
import pytest

import coracle
import mcd_oracle as O
from mcd import _lib, engine
from _gpu_util import gpu_tables, host_copies, input_par

pytestmark = pytest.mark.gpu

SI = input_par("Si", 10000.0, 1000.0, 0.0)
CU_CONT = input_par("Cu", 20000.0, 1000.0, 70.0, mode="cont", bethe="JL")
INT_KEYS = ("none", "bks", "abs", "trsm", "trdf", "long", "events", "double_rows", "nan_events")
INLINE = _lib.Tune(256, 0, 1, 2, 0)


@pytest.mark.parametrize("p", [SI, CU_CONT], ids=["ds", "cont"])
def test_empty_simulation(p):
    g = engine.run(p, num_el=0, seed=1)
    assert g.status == 0
    for k in INT_KEYS:
        assert g.tally[k] == 0, k
    assert g.tally["hist_E"].sum() == 0


def test_empty_simulations_inside_a_batch():
    sims = [dict(SI, num_el=0), dict(SI, num_el=500), dict(CU_CONT, num_el=0), dict(CU_CONT, num_el=300)]
    b = engine.Batch(sims, seed=9)
    res, status = b.run(INLINE)
    assert status == 0
    for k in INT_KEYS:
        assert res[0][k] == 0 and res[2][k] == 0, k
    for k, s in ((1, sims[1]), (3, sims[3])):
        sim = engine.make_sim(s, s["num_el"], seed=9, sim_id=k)
        mat = _lib.material(s["material"])
        tabs = gpu_tables(s) if engine.mode_of(s) == _lib.MODE_DS else None
        bufs = engine.RunBuffers(s["num_el"], _lib.FP32, False, 0)
        bufs.zero()
        engine.launch(sim, mat, tabs, bufs)
        ref = engine.collect(bufs).tally
        for key in INT_KEYS:
            assert res[k][key] == ref[key], (k, key)


def test_largest_batch():
    """256 simulations (the documented maximum) of every material, energy and
    mode; each simulation's electrons are all accounted for."""
    mats = ("Al", "Si", "Cu", "Au")
    sims = []
    for k in range(256):
        m = mats[k % 4]
        E0 = (5000.0, 10000.0, 20000.0, 30000.0)[(k // 4) % 4]
        tilt = (0.0, 20.0, 45.0, 70.0)[(k // 16) % 4]
        mode = "DS" if (k // 64) % 2 == 0 else "cont"
        sims.append(dict(input_par(m, E0, 1000.0, tilt, mode=mode, bethe="JL"), num_el=16 + k))
    b = engine.Batch(sims, seed=3)
    for t in (None, INLINE):
        res, status = b.run(t)
        assert status == 0
        for r, s in zip(res, sims):
            assert sum(r[o] for o in ("bks", "abs", "trsm", "trdf", "long")) == s["num_el"]
    assert _lib.lib().mcd_batch_workspace_bytes(256) > 0
    assert _lib.lib().mcd_batch_workspace_bytes(257) == 0


def _pair64(p, n, seed, first=0, **kw):
    g = engine.run(p, num_el=n, seed=seed, precision="fp64", first_electron=first)
    mat = O.Material(p["material"])
    ds = "DS" in p["mode"]
    c = coracle.run(mat, p["E0"], p["Emin"], p["s_tilt"], n, seed=seed, first=first, mode="DS" if ds else "cont",
                    Wc=p["Wc"], tables=host_copies(gpu_tables(p)) if ds else None,
                    bethe=p.get("Bethe_model", "classical"), thickness=float(p.get("thickness", 1e30)),
                    max_scatt=int(p.get("maxScatt", 10 ** 6)), **kw)
    return g, c


def _same(g, c, frac=0.99):
    e = g.electrons
    same = (e["outcome"] == c["outcome"]) & (e["n_events"] == c["n_events"])
    assert same.mean() >= frac, same.mean()


def test_event_limit_gives_long_rows():
    p = dict(SI, maxScatt=5)
    g, c = _pair64(p, 400, seed=2)
    _same(g, c, 1.0)
    t = g.tally
    assert t["long"] > 0.9 * 400
    assert t["events"] <= 5 * 400
    assert t["bks"] + t["abs"] + t["trsm"] + t["long"] == 400


def test_thin_film_transmits_on_first_step():
    p = dict(SI, thickness=1e-3)
    g, c = _pair64(p, 300, seed=5)
    _same(g, c, 1.0)
    assert g.tally["trsm"] == 300
    assert np.all(g.electrons["n_events"] == 1)


def test_beam_just_above_emin():
    p = input_par("Al", 1000.5, 1000.0, 0.0, mode="cont", bethe="JL")
    g, c = _pair64(p, 300, seed=6)
    _same(g, c)
    assert g.tally["abs"] + g.tally["bks"] == 300


def test_electron_indices_above_two_to_the_32():
    first = (1 << 40) + 12345
    g, c = _pair64(SI, 300, seed=8, first=first)
    _same(g, c)
    g0 = engine.run(SI, num_el=300, seed=8, precision="fp64", first_electron=0)
    # a different counter range draws different electrons
    assert not np.array_equal(g.electrons["n_events"], g0.electrons["n_events"])


@pytest.mark.parametrize("prec", ["fp32", "fp64"])
def test_block_size_does_not_change_results(prec):
    """Blocks of 1 to 16 threads (what a small job gets automatically) give
    the trajectories of full-warp blocks; other sizes are rejected."""
    runs = [engine.run(SI, num_el=300, seed=4, precision=prec, block_size=b) for b in (8, 1, 2, 4, 16, 32, 128, 0)]
    for g in runs[1:]:
        for k in INT_KEYS:
            assert g.tally[k] == runs[0].tally[k], k
        assert np.array_equal(g.electrons["n_events"], runs[0].electrons["n_events"])
        assert np.array_equal(g.electrons["final_E"], runs[0].electrons["final_E"])
    for b in (3, 24, 48, 512):
        with pytest.raises(_lib.MCDError):
            engine.run(SI, num_el=10, seed=4, precision=prec, block_size=b)
