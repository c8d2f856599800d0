"""Event streaming through double-buffered device rings (mcd.stream).

The records streamed chunk by chunk equal those of one run that captures
every event in a single ring (same Philox electron indices), and a ring too
small for a chunk is grown and the chunk re-run exactly.  Record-for-record
equality with the plain kernel needs the batched kernel's inline cross
sections (tune variant bit 1)."""
import numpy as np
import pytest

from mcd import _lib, engine
from mcd.stream import EventStream
from _gpu_util import input_par

pytestmark = pytest.mark.gpu

P = dict(input_par("Si", 10000.0, 1000.0, 0.0), num_el=12000)
INLINE = _lib.Tune(256, 0, 1, 2, 0)


def collect_stream(es):
    parts = []

    def consumer(rec, c):
        r = rec.copy()
        r["electron"] += c * es.chunk
        parts.append(r)

    stats = es.run(consumer)
    return np.concatenate(parts), stats


def key(rec):
    return rec[np.lexsort((rec["step_chan"] >> 5, rec["electron"]))]


@pytest.fixture(scope="module")
def single():
    g = engine.run(P, num_el=P["num_el"], seed=21, precision="fp32", ring_capacity=P["num_el"] * 1500)
    assert g.events_total <= P["num_el"] * 1500
    return key(g.events), g


def test_stream_equals_single_ring(single):
    ref, g = single
    es = EventStream(P, chunk=4000, seed=21, events_per_electron=450.0, tune=INLINE)
    rec, stats = collect_stream(es)
    assert stats["events"] == stats["events_tallied"] == rec.size == ref.size
    assert stats["reruns"] == 0
    rec = key(rec)
    for f in ("electron", "step_chan", "E", "W", "pathl", "c2", "half_phi", "x", "y", "z"):
        assert np.array_equal(rec[f], ref[f]), f
    assert stats["bytes"] == rec.size * 40


def test_stream_regrows_ring_exactly(single):
    ref, _ = single
    es = EventStream(P, chunk=6000, seed=21, ring_events=100000, piece_bytes=1 << 22, tune=INLINE)
    rec, stats = collect_stream(es)
    assert stats["reruns"] >= 1
    assert rec.size == ref.size
    assert np.array_equal(key(rec)["W"], ref["W"])


def test_stream_with_tables_delivers_every_tallied_event(single):
    ref, _ = single
    es = EventStream(P, chunk=4000, seed=21, events_per_electron=450.0)
    rec, stats = collect_stream(es)
    assert stats["events"] == stats["events_tallied"] == rec.size
    assert abs(rec.size - ref.size) <= 1e-3 * ref.size
    # every electron's steps arrive complete and in order 0..n-1
    rec = key(rec)
    steps = rec["step_chan"] >> 5
    first = np.r_[True, rec["electron"][1:] != rec["electron"][:-1]]
    assert np.all(steps[first] == 0)
    assert np.all(np.diff(steps)[~first[1:]] == 1)


def test_stream_of_selected_columns_equals_full_records(single):
    """Records carrying only step length, W, cos^2(theta/2) and position (the
    scatter_output columns of the streamed Au configuration) hold the same
    values as the full records."""
    ref, _ = single
    fields = _lib.EV_PATHL | _lib.EV_W | _lib.EV_C2 | _lib.EV_POS
    es = EventStream(P, chunk=4000, seed=21, events_per_electron=450.0, tune=INLINE, fields=fields)
    rec, stats = collect_stream(es)
    assert rec.dtype.itemsize == 32 and stats["bytes"] == rec.size * 32
    assert rec.size == ref.size
    rec = key(rec)
    for f in ("electron", "step_chan", "W", "pathl", "c2", "x", "y", "z"):
        assert np.array_equal(rec[f], ref[f]), f


def test_packed_header_stream_equals_full_records(single):
    """With the one-word header (electron << 4 | channel) a record of step
    length, W, cos^2(theta/2) and position is 28 bytes; the event index comes
    back from the ring order of each electron's records."""
    ref, _ = single
    fields = _lib.EV_PATHL | _lib.EV_W | _lib.EV_C2 | _lib.EV_POS | _lib.EV_PACKED_HEAD
    es = EventStream(P, chunk=4000, seed=21, events_per_electron=450.0, tune=INLINE, fields=fields,
                     piece_bytes=1 << 22)
    chunks = {}

    def consumer(rec, c):
        chunks.setdefault(c, []).append(rec.copy())

    stats = es.run(consumer)
    assert es.rec_bytes == 28 and stats["bytes"] == stats["events"] * 28
    parts = []
    for c in sorted(chunks):
        u = engine.unpack_events(np.concatenate(chunks[c]), fields)
        u["electron"] += c * es.chunk
        parts.append(u)
    rec = key(np.concatenate(parts))
    assert rec.size == ref.size
    for f in ("electron", "step_chan", "W", "pathl", "c2", "x", "y", "z"):
        assert np.array_equal(rec[f], ref[f]), f


def test_packed_header_single_ring_equals_full_records(single):
    ref, _ = single
    fields = _lib.EV_ALL | _lib.EV_PACKED_HEAD
    g = engine.run(P, num_el=P["num_el"], seed=21, precision="fp32", ring_capacity=P["num_el"] * 1500,
                   ring_fields=fields)
    rec = key(g.events)
    assert rec.size == ref.size
    for f in ("electron", "step_chan", "E", "W", "pathl", "c2", "half_phi", "x", "y", "z"):
        assert np.array_equal(rec[f], ref[f]), f


def test_consumer_exception_ends_the_run_and_the_stream_recovers(single):
    """A consumer that raises ends the run with its exception, after the work
    in flight has finished; the same stream then runs to completion."""
    ref, _ = single
    es = EventStream(P, chunk=4000, seed=21, events_per_electron=450.0, tune=INLINE, piece_bytes=1 << 22)

    class Stop(Exception):
        pass

    def bad(rec, c):
        if c == 1:
            raise Stop()

    with pytest.raises(Stop):
        es.run(bad)
    rec, stats = collect_stream(es)
    assert stats["events"] == stats["events_tallied"] == rec.size == ref.size
    rec = key(rec)
    assert np.array_equal(rec["W"], ref["W"]) and np.array_equal(rec["electron"], ref["electron"])
