"""The Python examples of the integration guide, at small sizes: a batch
with per-electron rows run through the autotuner and a CUDA graph, an event
stream with packed records, and the adjoint model through autograd."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_batch_stream_and_gradient_examples(tmp_path, monkeypatch):
    import torch

    import mcd
    from mcd import autotune
    from mcd.adjoint import ExitEnergyModel, exit_histogram
    from mcd.stream import EventStream

    monkeypatch.setenv("MCD_CACHE_DIR", str(tmp_path))
    sims = [dict(material=m, E0=E0, Emin=1000.0, s_tilt=t, Wc=100.0, tol_E=1e-3, tol_W=1e-3,
                 mode="DS", num_el=2000) for m in ("Al", "Cu") for E0 in (10e3, 20e3) for t in (0.0, 70.0)]
    batch = mcd.Batch(sims, seed=1, electrons=True)
    tune, _ = autotune.tune(batch, fraction=0.25, reps=1, blocks=(256, 1024), refills=(1, 4))
    graph = autotune.BatchGraph(batch, tune)
    graph.replay()
    tallies, status = batch.collect()
    rows = batch.electrons(3)
    assert len(tallies) == 8 and rows["outcome"].size == 2000
    assert (rows["outcome"] == 1).sum() == tallies[3]["bks"]
    assert rows["n_events"].sum() == tallies[3]["events"]

    got = [0]
    es = EventStream(dict(sims[0], num_el=3000), chunk=1000, fields=mcd._lib.EV_PACKED_HEAD,
                     events_per_electron=450.0)
    st = es.run(lambda records, chunk: got.__setitem__(0, got[0] + records.size))
    assert got[0] == st["events"] == st["events_tallied"] and es.rec_bytes == 36

    model = ExitEnergyModel(dict(material="Al", E0=15e3, Emin=1e3, s_tilt=70.0, mode="cont",
                                 Bethe_model="classical"), num_el=20000)
    J = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    n = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    h, mean = exit_histogram(J, n, model)
    (h.sum() + mean / 1e4).backward()
    assert np.isfinite(J.grad.item()) and np.isfinite(n.grad.item()) and J.grad.item() != 0.0
