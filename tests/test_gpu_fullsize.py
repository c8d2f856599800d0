"""The benchmarked workload at its full size (64 DS simulations, 8,927,966
electrons, about 5.5e9 events) through the batched kernel in the
benchmark's configuration, checked by properties that hold at any size:
  * every electron ends exactly once (bks + abs + trsm + trdf + long =
    num_el for every simulation) and nothing is flagged but NaN angles;
  * shards: the electrons of every simulation split at index F into
    [0, F) and [F, num_el), run as two batches on the same Philox electron
    indices, sum to the unsharded run -- integer counts, channel counts and
    histograms exactly, FP64 sums to rounding (the ranks of a multi-GPU run
    rely on this);
  * a relaunch of the same batch gives the same integer tallies."""
import pytest

import bench
from mcd import _lib, engine, shard
from _gpu_util import BENCH_TUNE

pytestmark = pytest.mark.gpu

SPLIT = 3000      # the smallest simulations (1000 electrons) fall wholly in the first shard


def run(sims, first=0):
    b = engine.Batch(sims, seed=0, first_electron=first, tally_channels=True)
    tallies, status = b.run(_lib.Tune(*BENCH_TUNE))
    assert status & ~_lib.FLAG_NAN == 0, status
    return b, tallies


@pytest.fixture(scope="module")
def full():
    sims = bench.workload()
    b, tallies = run(sims)
    return sims, b, tallies


def test_every_electron_ends_once(full):
    sims, _, tallies = full
    assert sum(s["num_el"] for s in sims) == 8_927_966
    for s, t in zip(sims, tallies):
        assert t["bks"] + t["abs"] + t["trsm"] + t["trdf"] + t["long"] == s["num_el"]
        assert t["none"] == 0 and t["long"] == 0 and t["trsm"] == 0 and t["trdf"] == 0
        assert int(t["hist_E"].sum()) <= t["bks"]          # energies of 20 keV and above fall outside
    assert sum(t["events"] for t in tallies) > 5e9


def test_two_shards_sum_to_the_whole(full):
    sims, _, whole = full
    head = [dict(s, num_el=min(s["num_el"], SPLIT)) for s in sims]
    tail = [dict(s, num_el=s["num_el"] - min(s["num_el"], SPLIT)) for s in sims]
    assert any(s["num_el"] == 0 for s in tail) and any(s["num_el"] > 0 for s in tail)
    _, ta = run(head)
    _, tb = run(tail, first=SPLIT)
    for k, (w, a, b) in enumerate(zip(whole, ta, tb)):
        m = shard.merge_tallies([a, b])
        for key in shard.INT_KEYS:
            assert m[key] == w[key], (k, key)
        for key in shard.ARRAY_KEYS:
            assert (m[key] == w[key]).all(), (k, key)
        for key in shard.SUM_KEYS:
            assert m[key] == pytest.approx(w[key], rel=1e-12, abs=1e-9), (k, key)


def test_relaunch_gives_the_same_tallies(full):
    _, b, first = full
    again, status = b.run(_lib.Tune(*BENCH_TUNE))
    assert status & ~_lib.FLAG_NAN == 0
    for w, a in zip(first, again):
        for key in shard.INT_KEYS:
            assert a[key] == w[key], key
        for key in shard.ARRAY_KEYS:
            assert (a[key] == w[key]).all(), key


def test_streamed_au_run_delivers_every_event_once():
    """The streamed configuration at its full size (Au 30 keV, tilt 70 deg,
    Wc 50 eV, tol 1e-4, 1e7 electrons in ten chunks, 28-byte packed records,
    about 9.2e9 events): each chunk delivers exactly the events its tallies
    count, every header names an electron of its chunk, and every record
    holds a positive step, a non-negative loss and a position inside the
    sample (these values checked in one 1 GB piece of four, to keep the host
    side short)."""
    import numpy as np
    from mcd.stream import EventStream
    p = dict(material="Au", E0=30000.0, Emin=500.0, s_tilt=70.0, Wc=50.0, tol_E=1e-4, tol_W=1e-4, mode="DS",
             num_el=10_000_000)
    fields = _lib.EV_PATHL | _lib.EV_W | _lib.EV_C2 | _lib.EV_POS | _lib.EV_PACKED_HEAD
    es = EventStream(p, chunk=1_000_000, seed=3, events_per_electron=950.0, fields=fields)
    seen = np.zeros(es.nchunks, dtype=np.int64)
    bad, pieces = [], [0]

    def consumer(rec, c):
        seen[c] += rec.size
        if (rec["head"] >> 4).max() >= es.chunk:
            bad.append((c, "electron"))
        pieces[0] += 1
        if pieces[0] % 4 == 1 and not ((rec["pathl"] > 0).all() and (rec["W"] >= 0).all() and (rec["z"] >= 0).all()):
            bad.append((c, "values"))

    st = es.run(consumer)
    assert not bad, bad[:5]
    per_chunk = np.array([t["events"] for t in st["tallies"]], dtype=np.int64)
    assert (seen == per_chunk).all()
    assert st["events"] == st["events_tallied"] == int(per_chunk.sum()) > 9e9
    assert sum(t["bks"] + t["abs"] + t["trsm"] + t["trdf"] + t["long"] for t in st["tallies"]) == p["num_el"]
