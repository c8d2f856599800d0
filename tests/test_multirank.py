"""Two ranks over gloo on CPU: each transports its contiguous share of the
electrons (the C oracle stands in for the GPU transport, which this host does
not have), the integer tallies are summed with one collective, and the result
equals a single-process run exactly, because the stream is counter-based."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as tmp

from mcd import shard

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _counts(res):
    oc = res["outcome"]
    t = {k: 0 for k in shard.INT_KEYS}
    for code, name in enumerate(("none", "bks", "abs", "trsm", "trdf", "long")):
        t[name] = int((oc == code).sum())
    t["events"] = int(res["n_events"].sum())
    t["double_rows"] = int((res["flags"] & 1).sum())
    t["channel"] = res["channel"].astype(np.int64)
    t["hist_E"] = np.bincount(np.minimum((res["final_E"][oc == 1] / 100.0).astype(int), 255), minlength=256)
    t["hist_T"] = np.zeros(180, np.int64)
    for k in shard.SUM_KEYS:
        t[k] = 0.0
    return t


def _run(first, n):
    import sys
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import coracle
    import mcd_oracle as O
    mat = O.Material("Al")
    T = np.load(os.path.join(ROOT, "tests", "golden", "tables.npz"))
    hts = [coracle.HostTable.build(k, mat, T["cfg4_Al_5/" + k + "/Ws"], T["cfg4_Al_5/" + k + "/Es"])
           for k in ("Moller", "Gryz")]
    return coracle.run(mat, 5000.0, 1000.0, 0.0, n, seed=3, first=first, mode="DS", Wc=100.0, tables=hts,
                       nthreads=2)


def _worker(rank, world, port, n, out_path):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    first, cnt = shard.shard_range(n, world, rank)
    t = _counts(_run(first, cnt))
    v = torch.from_numpy(shard.tally_vector(t))
    dist.all_reduce(v, op=dist.ReduceOp.SUM)
    if rank == 0:
        np.save(out_path, v.numpy())
    dist.barrier()
    dist.destroy_process_group()


def _tally(seed):
    rng = np.random.default_rng(seed)
    t = {k: int(rng.integers(0, 1000)) for k in shard.INT_KEYS}
    t.update({k: float(rng.uniform(0, 1e6)) for k in shard.SUM_KEYS})
    t.update(channel=rng.integers(0, 100, 16), hist_E=rng.integers(0, 100, 256), hist_T=rng.integers(0, 100, 180))
    return t


def _allreduce_worker(rank, world, port, out_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    got = shard.allreduce_tallies([_tally(10 * rank + k) for k in range(3)], dist)
    if rank == 0:
        np.save(out_path, np.array([np.concatenate([shard.tally_vector(t), [t[k] for k in shard.SUM_KEYS]])
                                    for t in got], dtype=np.float64))
    dist.barrier()
    dist.destroy_process_group()


def test_allreduce_tallies_sums_every_simulation(tmp_path):
    """The bench's whole-job counts under torchrun: every simulation's tally
    summed over two gloo ranks equals the host-side merge of the ranks'
    tallies."""
    out = str(tmp_path / "sums.npy")
    tmp.start_processes(_allreduce_worker, args=(2, _free_port(), out), nprocs=2, join=True, start_method="spawn")
    got = np.load(out)
    for k in range(3):
        m = shard.merge_tallies([_tally(k), _tally(10 + k)])
        want = np.concatenate([shard.tally_vector(m), [m[key] for key in shard.SUM_KEYS]])
        assert np.array_equal(got[k][:-3], want[:-3]), k
        assert np.allclose(got[k][-3:], want[-3:], rtol=1e-15), k


def test_shard_ranges_cover_exactly():
    n = 1001
    got = [shard.shard_range(n, 3, r, first=7) for r in range(3)]
    assert got[0][0] == 7
    assert sum(c for _, c in got) == n
    for (a, ca), (b, _) in zip(got, got[1:]):
        assert a + ca == b
    with pytest.raises(ValueError):
        shard.shard_range(10, 2, 2)


def test_two_gloo_ranks_equal_single_process(tmp_path):
    n = 2000
    out = str(tmp_path / "sum.npy")
    tmp.start_processes(_worker, args=(2, _free_port(), n, out), nprocs=2, join=True, start_method="spawn")
    merged = shard.tally_from_vector(np.load(out))
    single = _counts(_run(0, n))
    for k in shard.INT_KEYS:
        assert merged[k] == single[k], k
    for k in ("channel", "hist_E"):
        assert np.array_equal(merged[k], single[k]), k


def test_merge_tallies():
    a = {k: 1 for k in shard.INT_KEYS}
    a.update({k: 0.5 for k in shard.SUM_KEYS})
    a.update(channel=np.ones(16, np.int64), hist_E=np.ones(256, np.int64), hist_T=np.ones(180, np.int64))
    m = shard.merge_tallies([a, a, a])
    assert m["bks"] == 3 and m["sum_E_bks"] == 1.5 and m["hist_E"].sum() == 768
    assert shard.replica_offset(3) == 3 << 40
