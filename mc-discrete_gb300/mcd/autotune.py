"""Launch tuning of the batched persistent kernel, and its CUDA graph.

tune(batch) times the kernel on a scaled-down copy of the batch (every
simulation keeps its parameters; electron counts shrink) for each block size
x refill granularity x register budget, times the few fastest again on the
batch itself, and returns the fastest mcd_tune.  Results are cached
in a JSON file keyed by the GPU name and a signature of the workload, so a
later process reuses them without timing.

BatchGraph(batch, tune) captures one step (zero the tallies and status, reset
the work queue, launch) in a CUDA graph; replay() runs it with one call.
"""
import hashlib
import json
import os

from . import _lib
from .engine import Batch, _torch

BLOCKS = (128, 256, 512, 576, 1024)
LOWREG_MAX_BLOCK = 576     # the 56-register kernel (tune variant bit 0), two blocks per SM
REFILLS = (1, 2, 4, 8, 16)


def _cache_path():
    base = os.environ.get("MCD_CACHE_DIR") or os.path.join(os.path.expanduser("~"), ".cache", "mcd")
    return os.path.join(base, "autotune.json")


def signature(batch):
    """Workload signature: what changes the best launch shape."""
    torch = _torch()
    parts = [torch.cuda.get_device_name(batch.device)]
    for p in batch.inputs:
        parts.append("%s/%s/%g/%g/%g/%d" % (p["material"], p["mode"], p["E0"], p["Emin"], p["s_tilt"],
                                           len(str(int(p["num_el"])))))
    return hashlib.sha1("|".join(parts).encode()).hexdigest()[:16]


def _load():
    try:
        with open(_cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(db):
    path = _cache_path()
    try:
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(db, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    except OSError:
        pass


def _time(batch, t, reps):
    torch = _torch()
    st = torch.cuda.current_stream(batch.device)
    batch.zero()
    batch.launch(t)                     # warm-up of this shape
    best = float("inf")
    for _ in range(reps):
        batch.zero()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(st)
        batch.launch(t)
        b.record(st)
        torch.cuda.synchronize(batch.device)
        best = min(best, a.elapsed_time(b))
    return best


def tune(batch, fraction=0.1, reps=2, use_cache=True, blocks=BLOCKS, refills=REFILLS, finalists=3):
    """Fastest mcd_tune for `batch`; returns (tune, table of timings in ms).
    Every shape is timed on the scaled-down copy; the `finalists` fastest,
    and the fastest refill of every (block size, register budget) pair, are
    timed again on the batch itself, which decides."""
    key = signature(batch)
    db = _load() if use_cache else {}
    if key in db:
        c = db[key]
        return _lib.Tune(c["block"], 0, c["refill"], c.get("variant", 0), 0), c.get("table", {})
    sims = [dict(p, num_el=max(64, int(round(p["num_el"] * fraction)))) for p in batch.inputs]
    probe = Batch(sims, seed=12345, device=batch.device)
    table = {}
    best = None
    for b in blocks:
        for r in refills:
            for v in ((0, 1) if b <= LOWREG_MAX_BLOCK else (0,)):
                t = _lib.Tune(b, 0, r, v, 0)
                try:
                    ms = _time(probe, t, reps)
                except _lib.MCDError:
                    continue
                table["%d/%d/%d" % (b, r, v)] = ms
                if best is None or ms < best[0]:
                    best = (ms, b, r, v)
    if best is None:
        raise RuntimeError("no launch shape fits the batched kernel")
    if finalists > 1:
        # each (block size, register budget) pair sends its fastest refill on
        # the copy and refill 1, with the `finalists` fastest shapes overall,
        # to be timed on the batch itself.  The copy's short run (about 5
        # electrons per thread against about 57 on the full 64-simulation
        # workload) is ruled by its tail and misranks shapes: it puts
        # 1024/1/0 at 10.0 ms and 576/1/1 at 10.7 ms, and prefers refill 2
        # for blocks of 576, where the batch itself takes 79.1, 78.2 and
        # 79.1 ms (576/2/1).
        order = sorted(table.items(), key=lambda kv: kv[1])
        ranked = order[:finalists]
        seen = set()
        for k, ms in order:
            b, r, v = k.split("/")
            pick = (b, v) not in seen or r == "1"
            seen.add((b, v))
            if pick and (k, ms) not in ranked:
                ranked.append((k, ms))
        full = []
        for k, _ in ranked:
            b, r, v = (int(x) for x in k.split("/"))
            full.append((_time(batch, _lib.Tune(b, 0, r, v, 0), 3), b, r, v))
            table["full:" + k] = full[-1][0]
        best = min(full)
    db[key] = {"block": best[1], "refill": best[2], "variant": best[3], "table": table}
    if use_cache:
        _store(db)
    return _lib.Tune(best[1], 0, best[2], best[3], 0), table


class BatchGraph:
    """One batched step captured in a CUDA graph."""

    def __init__(self, batch, tune_params):
        torch = _torch()
        self.batch = batch
        self.tune = tune_params
        # one eager step first: the launch configures the kernel outside capture
        batch.zero()
        batch.launch(tune_params)
        torch.cuda.synchronize(batch.device)
        self.graph = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(batch.device)
        s.wait_stream(torch.cuda.current_stream(batch.device))
        with torch.cuda.stream(s):
            with torch.cuda.graph(self.graph, stream=s):
                batch.zero()
                batch.launch(tune_params)
        torch.cuda.current_stream(batch.device).wait_stream(s)

    def replay(self):
        self.graph.replay()

    def run(self):
        self.replay()
        return self.batch.collect()
