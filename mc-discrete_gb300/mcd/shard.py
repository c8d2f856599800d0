"""Splitting electrons across GPUs (one process per GPU).

Every electron owns its Philox counter range (event, electron index, sim), so
a simulation split into contiguous index ranges gives exactly the electrons a
single process would: there is no data exchange while transporting, and the
only exchange is one sum of the integer/FP64 tallies at the end.
"""
import numpy as np

from . import _lib

INT_KEYS = ("none", "bks", "abs", "trsm", "trdf", "long", "events", "double_rows", "nan_events",
            "clamped", "long_path", "table_range")
SUM_KEYS = ("sum_E_bks", "sum_E2_bks", "sum_steps2")
ARRAY_KEYS = ("channel", "hist_E", "hist_T")


def shard_range(num_el, world, rank, first=0):
    """(first electron index, count) of `rank`'s contiguous share."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad world/rank")
    lo = num_el * rank // world
    hi = num_el * (rank + 1) // world
    return first + lo, hi - lo


def replica_offset(rank, bits=40):
    """First electron index of a replica that runs the whole workload on its
    own indices (weak scaling): 2^40 electrons apart."""
    return int(rank) << bits


def merge_tallies(tallies):
    """Sum per-shard tally dicts (as returned by mcd.engine) into one."""
    out = {}
    for k in INT_KEYS:
        out[k] = int(sum(t[k] for t in tallies))
    for k in SUM_KEYS:
        out[k] = float(sum(t[k] for t in tallies))
    for k in ARRAY_KEYS:
        out[k] = np.sum([np.asarray(t[k], dtype=np.int64) for t in tallies], axis=0)
    return out


def tally_vector(t):
    """Flatten the integer part of a tally for a collective sum."""
    return np.concatenate([[t[k] for k in INT_KEYS]] + [np.asarray(t[k], dtype=np.int64) for k in ARRAY_KEYS])


def tally_from_vector(v, sums=None):
    v = np.asarray(v, dtype=np.int64)
    out = {k: int(v[i]) for i, k in enumerate(INT_KEYS)}
    o = len(INT_KEYS)
    for k, n in zip(ARRAY_KEYS, (_lib.MAX_CHANNELS, _lib.HIST_E_MAX, _lib.HIST_T_MAX)):
        out[k] = v[o:o + n].copy()
        o += n
    for k in SUM_KEYS:
        out[k] = float(sums[k]) if sums else 0.0
    return out


def allreduce_tallies(tallies, dist, device=None):
    """The per-simulation tallies of this rank summed over every rank of the
    default process group (torch.distributed): one all-reduce of the integer
    counts (tally_vector) and one of the FP64 sums, on `device` (the rank's
    GPU under NCCL; None keeps them on the host, as gloo wants)."""
    import torch
    v = torch.from_numpy(np.stack([tally_vector(t) for t in tallies]).astype(np.int64))
    s = torch.tensor([[float(t[k]) for k in SUM_KEYS] for t in tallies], dtype=torch.float64)
    if device is not None:
        v, s = v.to(device), s.to(device)
    dist.all_reduce(v)
    dist.all_reduce(s)
    return [tally_from_vector(a, dict(zip(SUM_KEYS, b))) for a, b in zip(v.cpu().numpy(), s.cpu().numpy())]
