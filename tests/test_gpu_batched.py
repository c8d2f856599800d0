"""The batched persistent kernel against one plain launch per simulation.

With inline cross sections (tune variant bit 1) both run the same event code
on the same Philox counters (sim id, electron, event), so the integer tallies
must agree; the refill setting only changes which lane runs which electron,
never the result.  The default tabulated cross sections differ from the
inline ones by at most 3e-7 relative, which moves a handful of trajectories:
their tallies are checked against the inline ones within that allowance,
and a plain launch reading the same table (mcd_sim.sigma_table) matches
the batched kernel exactly."""
import numpy as np
import pytest

from mcd import _lib, engine
from _gpu_util import input_par

pytestmark = pytest.mark.gpu

SIMS = [
    dict(input_par("Si", 10000.0, 1000.0, 0.0), num_el=3000),
    dict(input_par("Au", 20000.0, 1000.0, 45.0), num_el=700),
    dict(input_par("Cu", 5000.0, 1000.0, 70.0), num_el=5000),
    dict(input_par("Al", 30000.0, 1000.0, 20.0), num_el=1200),
    dict(input_par("Cu", 20000.0, 1000.0, 70.0, mode="cont", bethe="JL"), num_el=2500),
    dict(input_par("Al", 15000.0, 1000.0, 70.0, mode="cont", bethe="classical"), num_el=64),
    dict(input_par("Si", 10000.0, 1000.0, 0.0, elastic="Ruth_nigram"), num_el=1500),
    dict(input_par("Si", 10000.0, 1000.0, 0.0, diffMFP=True, thickness=3000.0), num_el=2000),
]

INT_KEYS = ("none", "bks", "abs", "trsm", "trdf", "long", "events", "double_rows", "nan_events",
            "clamped", "long_path", "table_range")


def plain(k, p, tabulated=False):
    # the batched kernel uses sim id = index in the batch; match it here
    mat = _lib.material(p["material"])
    sim = engine.make_sim(p, p["num_el"], seed=42, sim_id=k)
    if tabulated:
        engine.use_sigma_table(sim, mat)
    tabs = None
    if engine.mode_of(p) == _lib.MODE_DS:
        from mcd.tables import ds_tables
        tabs = ds_tables(mat, p["E0"], p["Emin"], p["Wc"], p["tol_E"], p["tol_W"])
    bufs = engine.RunBuffers(p["num_el"], _lib.FP32, False, 0)
    bufs.zero()
    engine.launch(sim, mat, tabs, bufs)
    return engine.collect(bufs).tally


@pytest.fixture(scope="module")
def plain_tallies():
    return [plain(k, p) for k, p in enumerate(SIMS)]


@pytest.mark.parametrize("variant", [2, 3])
@pytest.mark.parametrize("refill", [1, 8, 32])
@pytest.mark.parametrize("block", [128, 256])
def test_batched_equals_plain(plain_tallies, refill, block, variant):
    b = engine.Batch(SIMS, seed=42)
    res, status = b.run(_lib.Tune(block, 0, refill, variant, 0))
    for k, (t, ref) in enumerate(zip(res, plain_tallies)):
        for key in INT_KEYS:
            assert t[key] == ref[key], (k, key, t[key], ref[key])
        assert np.array_equal(t["hist_E"], ref["hist_E"])
        assert np.array_equal(t["hist_T"], ref["hist_T"])
        assert abs(t["sum_E_bks"] - ref["sum_E_bks"]) <= 1e-9 * max(1.0, ref["sum_E_bks"])
        assert sum(t[o] for o in ("bks", "abs", "trsm", "trdf", "long")) == SIMS[k]["num_el"]


@pytest.mark.parametrize("variant", [0, 1])
def test_plain_with_its_table_equals_batched(variant):
    """mcd_build_sigma_table builds the table the batched path builds for a
    simulation whose group spans its own energy range (true of every DS
    simulation here), so a plain launch reading it runs the batched
    kernel's trajectories."""
    b = engine.Batch(SIMS, seed=42)
    res, status = b.run(_lib.Tune(256, 0, 1, variant, 0))
    for k, p in enumerate(SIMS):
        ref = plain(k, p, tabulated=True)
        for key in INT_KEYS:
            assert res[k][key] == ref[key], (k, key, res[k][key], ref[key])
        assert np.array_equal(res[k]["hist_E"], ref["hist_E"])


def test_batched_rows_equal_plain_rows():
    """A batch that keeps per-electron rows (mcd_sim.electrons) writes the
    rows a plain launch writes for the same electrons."""
    from mcd.tables import ds_tables
    b = engine.Batch(SIMS, seed=42, electrons=True)
    b.run(_lib.Tune(256, 0, 1, 0, 0))
    for k, p in enumerate(SIMS):
        mat = _lib.material(p["material"])
        sim = engine.make_sim(p, p["num_el"], seed=42, sim_id=k)
        engine.use_sigma_table(sim, mat)
        tabs = None
        if engine.mode_of(p) == _lib.MODE_DS:
            tabs = ds_tables(mat, p["E0"], p["Emin"], p["Wc"], p["tol_E"], p["tol_W"])
        bufs = engine.RunBuffers(p["num_el"], _lib.FP32, True, 0)
        bufs.zero()
        engine.launch(sim, mat, tabs, bufs)
        ref, got = engine.collect(bufs).electrons, b.electrons(k)
        for key in ("outcome", "flags", "n_events", "final_E", "dir", "last_pos", "max_z"):
            assert np.array_equal(got[key], ref[key], equal_nan=True), (k, key)


@pytest.mark.parametrize("variant", [0, 1])
def test_tabulated_cross_sections_follow_inline(variant):
    sims = [dict(p, num_el=4 * p["num_el"]) for p in SIMS]
    b = engine.Batch(sims, seed=21)
    inl, st_i = b.run(_lib.Tune(256, 0, 1, variant | 2, 0))
    tab, st_t = b.run(_lib.Tune(256, 0, 1, variant, 0))
    assert st_i == st_t == 0
    changed = 0
    for k, (t, r) in enumerate(zip(tab, inl)):
        n = sims[k]["num_el"]
        assert sum(t[o] for o in ("bks", "abs", "trsm", "trdf", "long")) == n
        for o in ("bks", "abs", "trsm", "trdf"):
            assert abs(t[o] - r[o]) <= 3 + 1e-3 * n, (k, o, t[o], r[o])
        assert abs(t["events"] - r["events"]) <= 1e-3 * r["events"], k
        assert np.abs(t["hist_E"].astype(np.int64) - r["hist_E"]).sum() <= 6 + 2e-3 * n, k
        changed += int(t["events"] != r["events"])
        if engine.mode_of(sims[k]) == _lib.MODE_CONT:
            # continuous-mode simulations never use the tables
            for key in INT_KEYS:
                assert t[key] == r[key], (k, key)
    # the tables are in use: DS simulations with many events do move
    assert changed >= 1


def test_batched_relaunch_is_identical():
    b = engine.Batch(SIMS[:4], seed=3)
    r1, _ = b.run()
    r2, _ = b.run()
    for t1, t2 in zip(r1, r2):
        for key in INT_KEYS:
            assert t1[key] == t2[key]


def test_batched_rejects_bad_tuning():
    b = engine.Batch(SIMS[:1], seed=3)
    with pytest.raises(_lib.MCDError):
        b.launch(_lib.Tune(100, 0, 1, 0, 0))
    with pytest.raises(_lib.MCDError):
        b.launch(_lib.Tune(128, 0, 40, 0, 0))


def test_graph_replay_equals_direct_launch():
    from mcd import autotune
    b = engine.Batch(SIMS, seed=8)
    t = _lib.Tune(256, 0, 1, 0, 0)
    ref, _ = b.run(t)
    g = autotune.BatchGraph(b, t)
    for _ in range(2):
        res, _ = g.run()
        for a, r in zip(res, ref):
            for key in INT_KEYS:
                assert a[key] == r[key], key


def test_autotune_picks_a_measured_shape(tmp_path, monkeypatch):
    from mcd import autotune
    monkeypatch.setenv("MCD_CACHE_DIR", str(tmp_path))
    b = engine.Batch(SIMS[:3], seed=4)
    t, table = autotune.tune(b, fraction=0.2, reps=1, blocks=(128, 256), refills=(1, 8))
    k = "%d/%d/%d" % (t.block_size, t.refill, t.variant)
    full = {key[5:]: ms for key, ms in table.items() if key.startswith("full:")}
    scaled = {key: ms for key, ms in table.items() if not key.startswith("full:")}
    # the finalists are the three fastest on the scaled copy and, for every
    # (block, register budget) pair, its fastest refill and refill 1; the
    # batch itself decides
    want = set(sorted(scaled, key=scaled.get)[:3])
    for b_ in (128, 256):
        for v in (0, 1):
            of = [key for key in scaled if key.startswith("%d/" % b_) and key.endswith("/%d" % v)]
            if of:
                want.add(min(of, key=scaled.get))
                want |= {key for key in of if key.split("/")[1] == "1"}
    assert set(full) == want
    assert k in full and min(full.values()) == full[k]
    t2, _ = autotune.tune(b)          # from the cache
    assert (t2.block_size, t2.refill) == (t.block_size, t.refill)
