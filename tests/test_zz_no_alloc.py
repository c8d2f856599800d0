"""The batched run that allocates nothing (mcd_run_batched_noalloc).

Callers that cannot call cudaMalloc (an application that owns all device
memory through its own arena, or one whose latency budget cannot absorb an
allocation that may synchronise the device) use this entry point: its
scratch lives in a static device array inside the library, and the caller
passes only inputs and outputs.  It must give the same tallies as the
workspace-based mcd_batch_prepare + mcd_run_batched, call after call, since
every call rewrites the shared array.

This file is named to be collected last; it also passes when run alone.
"""
import ctypes as C

import numpy as np
import pytest

from mcd import _lib, engine
from _gpu_util import input_par

pytestmark = pytest.mark.gpu

SIMS = [
    dict(input_par("Si", 10000.0, 1000.0, 0.0), num_el=2000),
    dict(input_par("Au", 20000.0, 1000.0, 45.0), num_el=500),
    dict(input_par("Cu", 5000.0, 1000.0, 70.0), num_el=3000),
    dict(input_par("Cu", 20000.0, 1000.0, 70.0, mode="cont", bethe="JL"), num_el=1500),
]

INT_KEYS = ("none", "bks", "abs", "trsm", "trdf", "long", "events", "double_rows", "nan_events",
            "clamped", "long_path", "table_range")


def _noalloc(b, tune):
    import torch
    tallies = torch.zeros_like(b.tallies)
    status = torch.zeros(1, dtype=torch.int32, device=b.device)
    st = torch.cuda.current_stream(b.device)
    code = _lib.lib().mcd_run_batched_noalloc(b._sims_arr, b.n, b.mats, b._idx[0], b._tarr, b._idx[1],
                                              b._idx[2], tallies.data_ptr(), C.byref(tune),
                                              status.data_ptr(), st.cuda_stream)
    _lib.check("mcd_run_batched_noalloc", code)
    host = tallies.cpu().numpy()
    return [engine.tally_from_bytes(host[k]) for k in range(b.n)], int(status.item())


def _same(a, b):
    for ta, tb in zip(a, b):
        for k in INT_KEYS:
            assert ta[k] == tb[k], k
        assert np.array_equal(ta["hist_E"], tb["hist_E"])
        assert np.array_equal(ta["hist_T"], tb["hist_T"])
        assert abs(ta["sum_E_bks"] - tb["sum_E_bks"]) <= 1e-9 * max(1.0, abs(tb["sum_E_bks"]))


def test_noalloc_matches_workspace_run_twice():
    # the no-alloc entry evaluates cross sections inline; so does variant bit 1
    tune = _lib.Tune(256, 0, 1, 2, 0)
    b = engine.Batch(SIMS, seed=17)
    ref, st_ref = b.run(tune)
    first, st1 = _noalloc(b, tune)
    second, st2 = _noalloc(b, tune)
    _same(first, ref)
    _same(second, ref)
    assert st1 == st2 == st_ref
    for t, s in zip(first, SIMS):
        assert sum(t[o] for o in ("bks", "abs", "trsm", "long")) == s["num_el"]


def test_noalloc_reads_caller_built_cross_section_tables():
    """Simulations that carry a table from mcd_build_sigma_table run from it;
    each DS simulation here is alone in its cross-section group, so the
    workspace run's tables are the same tables and the tallies agree."""
    b = engine.Batch(SIMS, seed=17)
    ref, st_ref = b.run(_lib.Tune(256, 0, 1, 0, 0))
    keep = [engine.use_sigma_table(b._sims_arr[k], b.mats[b._idx[0][k]]) for k in range(b.n)]
    assert sum(t is not None for t in keep) == 3
    got, st = _noalloc(b, _lib.Tune(256, 0, 1, 0, 0))
    _same(got, ref)
    assert st == st_ref


def test_noalloc_honours_the_tune_variant_bits():
    """Bit 1 evaluates the cross sections inline even for simulations that
    carry a caller-built table; bit 0 runs the 56-register kernel.  Both
    give the workspace run's tallies under the same bits."""
    b = engine.Batch(SIMS, seed=23)
    keep = [engine.use_sigma_table(b._sims_arr[k], b.mats[b._idx[0][k]]) for k in range(b.n)]
    assert sum(t is not None for t in keep) == 3
    for variant in (2, 3):
        tune = _lib.Tune(256, 0, 1, variant, 0)
        ref, st_ref = b.run(tune)          # the workspace ignores sigma_table: its own tables or inline
        got, st = _noalloc(b, tune)
        _same(got, ref)
        assert st == st_ref
    with pytest.raises(_lib.MCDError):
        _noalloc(b, _lib.Tune(640, 0, 1, 1, 0))     # the 56-register kernel takes at most 576 threads


def test_noalloc_at_its_limit_of_64_simulations():
    """Exactly MCD_STATIC_MAX_SIMS simulations fill the static array and the
    largest shared-memory layout; a few electrons each, two calls in a row,
    against the workspace run."""
    sims = []
    for k in range(_lib.STATIC_MAX_SIMS):
        m = ("Al", "Si", "Cu", "Au")[k % 4]
        E0 = (5000.0, 10000.0, 20000.0, 30000.0)[(k // 4) % 4]
        tilt = (0.0, 20.0, 45.0, 70.0)[k // 16]
        mode = "cont" if k % 9 == 4 else "DS"
        sims.append(dict(input_par(m, E0, 1000.0, tilt, mode=mode, bethe="JL"), num_el=3 + (k * 7) % 11))
    tune = _lib.Tune(256, 0, 1, 2, 0)
    b = engine.Batch(sims, seed=29)
    ref, st_ref = b.run(tune)
    for _ in range(2):
        got, st = _noalloc(b, tune)
        _same(got, ref)
        assert st == st_ref
    for t, s in zip(got, sims):
        assert sum(t[o] for o in ("bks", "abs", "trsm", "long")) == s["num_el"]


def test_noalloc_rejects_too_many_simulations():
    b = engine.Batch(SIMS[:1], seed=1)
    n = _lib.STATIC_MAX_SIMS + 1
    sims = (_lib.Sim * n)(*([b.structs[0]] * n))
    idx = (C.c_int32 * n)(*([0] * n))
    tg = (C.c_int32 * n)(*([1] * n))
    code = _lib.lib().mcd_run_batched_noalloc(sims, n, b.mats, idx, b._tarr, idx, tg, b.tallies.data_ptr(),
                                              None, b.status.data_ptr(), None)
    assert code == _lib.ETOOBIG
