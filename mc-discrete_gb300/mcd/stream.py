"""Streaming of per-event records (scatter_output) for runs too large to hold.

The reference appends every event to per-electron Python lists, pickles them
back to the parent process and appends them to an HDF5 store
(MC/tools/fileTools.py:193-242, MC/doScatter.py:99-119).  Here the electrons
of a simulation are cut into chunks; each chunk runs as one batched
persistent launch whose every event is appended to a device ring
(mcd_run_batched_ring), as a full 40-byte record or with only the fields a
field mask selects (the scatter_output columns wanted; 8-byte header plus
4 bytes per column, or a 4-byte header with EV_PACKED_HEAD, whose records
engine.unpack_events turns back into the 8-byte form chunk by chunk).  Two
rings alternate: while chunk c+1 is being transported, chunk c's records
are copied to pinned host memory on a second stream, in pieces handed to a
consumer callback; the copy of the next piece runs while the consumer reads
the current one.  A chunk whose events do
not fit its ring is re-run with a larger ring; the counter-based random
stream makes the re-run exact.
"""
import ctypes as C
import time

from . import _lib
from .config import with_defaults
from .engine import Batch, _torch, event_dtype


class EventStream:
    """Stream the events of one simulation through double-buffered device rings.

    input_par   input.file parameters (DS or continuous) with num_el
    chunk       electrons per launch (each chunk's electrons keep their own
                Philox indices, so the stream equals one big run)
    ring_events record capacity of each device ring (default: 1.3x the
                estimated events of a chunk, grown on overflow)
    piece_bytes size of each host copy handed to the consumer
    """

    def __init__(self, input_par, chunk=1_000_000, seed=0, ring_events=None, piece_bytes=1 << 30,
                 events_per_electron=None, tune=None, device="cuda", fields=0):
        torch = _torch()
        self.p = with_defaults(input_par)
        self.num_el = int(self.p["num_el"])
        self.chunk = int(min(chunk, self.num_el))
        self.seed = int(seed)
        self.fields = int(fields)
        self.dtype = event_dtype(self.fields)
        self.rec_bytes = self.dtype.itemsize
        self.device = torch.device(device)
        self.tune = tune if tune is not None else _lib.Tune(256, 0, 1, 0, 0)
        self.nchunks = (self.num_el + self.chunk - 1) // self.chunk
        # one prepared workspace per chunk (built once, so launches never wait on the host)
        self.batches = []
        for c in range(self.nchunks):
            first = c * self.chunk
            n = min(self.chunk, self.num_el - first)
            self.batches.append(Batch([dict(self.p, num_el=n)], seed=self.seed, device=self.device,
                                      first_electron=first))
        epe = events_per_electron or 1000.0
        cap = int(ring_events) if ring_events else int(1.3 * epe * self.chunk) + 4096
        self.piece = max(self.rec_bytes, (int(piece_bytes) // self.rec_bytes) * self.rec_bytes)
        self._alloc_rings(cap)
        self.host = [torch.empty(self.piece, dtype=torch.uint8, pin_memory=True) for _ in range(2)]
        self.copy_stream = torch.cuda.Stream(self.device)
        self.cursor_host = torch.zeros(2, dtype=torch.int64, pin_memory=True)

    def _alloc_rings(self, cap):
        torch = _torch()
        self.cap = int(cap)
        self.rings = [torch.empty(self.cap * self.rec_bytes, dtype=torch.uint8, device=self.device) for _ in range(2)]
        self.cursors = [torch.zeros(1, dtype=torch.int64, device=self.device) for _ in range(2)]

    def _launch(self, c, slot, stream):
        b = self.batches[c]
        b.tallies.zero_()
        b.status.zero_()
        self.cursors[slot].zero_()
        ring = _lib.EventRing(self.rings[slot].data_ptr(), self.cap, self.cursors[slot].data_ptr(), self.fields, 0)
        code = _lib.lib().mcd_run_batched_ring(b.ws_ptr, b.n, b.tallies.data_ptr(), C.byref(self.tune),
                                               C.byref(ring), b.status.data_ptr(), stream.cuda_stream)
        _lib.check("mcd_run_batched_ring", code)

    def run(self, consumer=None):
        """Transport every chunk; consumer(records, chunk_index) gets each host
        piece as a numpy structured array (a view valid during the call).
        Returns a dict with the event and byte counts and the wall time.  An
        exception raised by the consumer ends the run: the launches and copies
        in flight finish first, and the stream can be run again."""
        torch = _torch()
        try:
            return self._run(consumer)
        except BaseException:
            torch.cuda.synchronize(self.device)
            raise

    def _run(self, consumer):
        torch = _torch()
        cs = torch.cuda.current_stream(self.device)
        done = [torch.cuda.Event() for _ in range(2)]
        freed = [torch.cuda.Event() for _ in range(2)]
        copied = [torch.cuda.Event() for _ in range(2)]   # the last copy into each host buffer
        t0 = time.perf_counter()
        total_events = 0
        total_bytes = 0
        reruns = 0
        pending = []
        for c in range(min(2, self.nchunks)):
            self._launch(c, c % 2, cs)
            done[c % 2].record(cs)
            pending.append(c)
        c_next = len(pending)
        while pending:
            c = pending.pop(0)
            slot = c % 2
            with torch.cuda.stream(self.copy_stream):
                self.copy_stream.wait_event(done[slot])
                self.cursor_host[slot].copy_(self.cursors[slot][0], non_blocking=True)
            self.copy_stream.synchronize()
            n = int(self.cursor_host[slot])
            if n > self.cap:
                # the chunk's events did not fit: grow both rings, re-run this chunk
                # and relaunch the one queued behind it on the new rings
                reruns += 1
                torch.cuda.synchronize(self.device)
                self._alloc_rings(int(n * 1.2) + 4096)
                self._launch(c, slot, cs)
                done[slot].record(cs)
                pending.insert(0, c)
                if pending[1:]:
                    o = pending[1]
                    self._launch(o, o % 2, cs)
                    done[o % 2].record(cs)
                continue
            nbytes = n * self.rec_bytes
            ring = self.rings[slot]
            pieces = [(off, min(self.piece, nbytes - off)) for off in range(0, nbytes, self.piece)]

            def issue(j):
                # piece j into host buffer j % 2, whose previous piece the
                # consumer has already returned from
                off, k = pieces[j]
                with torch.cuda.stream(self.copy_stream):
                    self.host[j % 2][:k].copy_(ring[off:off + k], non_blocking=True)
                    copied[j % 2].record(self.copy_stream)

            if pieces:
                issue(0)
            for j, (_, k) in enumerate(pieces):
                if j + 1 < len(pieces):
                    issue(j + 1)            # the next piece crosses the link while the consumer reads this one
                copied[j % 2].synchronize()
                if consumer is not None:
                    consumer(self.host[j % 2][:k].numpy().view(self.dtype), c)
            with torch.cuda.stream(self.copy_stream):
                freed[slot].record(self.copy_stream)
            total_events += n
            total_bytes += nbytes
            if c_next < self.nchunks:
                cs.wait_event(freed[slot])
                self._launch(c_next, slot, cs)
                done[slot].record(cs)
                pending.append(c_next)
                c_next += 1
        torch.cuda.synchronize(self.device)
        wall = time.perf_counter() - t0
        tallies = [b.collect()[0][0] for b in self.batches]
        ev = sum(t["events"] for t in tallies)
        return {"events": total_events, "events_tallied": ev, "bytes": total_bytes, "wall_s": wall,
                "reruns": reruns, "tallies": tallies}
