"""Continuous-mode histogram workload: JL Bethe, Cu, 20 keV -> 1 keV, tilt
70 deg, 1e6 electrons, exit-energy tally of 200 x 100 eV bins and polar
exit-angle tally of 90 x 1 deg bins (the energy loss of
MC/tools/scattering.py:844-883 with the Joy-Luo law of
MC/tools/stoppingPowers.py:145-173).

The CUDA tallies (FP32 transport) are compared with histograms of the C
oracle's per-electron rows for the same electrons and the same Philox
stream: backscatter yield by a two-proportion z test, both histograms by a
chi-square homogeneity test; the persistent batched kernel's tallies equal
the plain kernel's bin for bin."""
import numpy as np
import pytest
from scipy import stats

import coracle
import mcd_oracle as O
from mcd import _lib, engine
from _gpu_util import eta_z, input_par

pytestmark = pytest.mark.gpu

P = input_par("Cu", 20000.0, 1000.0, 70.0, mode="cont", bethe="JL")
N = 1_000_000
SEED = 5


def binned(values, width, nbins):
    """Bin i holds [i * width, (i + 1) * width), as the device tallies do."""
    idx = np.floor(np.asarray(values, dtype=np.float64) / width)
    idx = idx[(idx >= 0) & (idx < nbins)].astype(np.int64)
    return np.bincount(idx, minlength=nbins)


@pytest.fixture(scope="module")
def runs():
    g = engine.run(P, num_el=N, seed=SEED, precision="fp32", electrons=False)
    c = coracle.run(O.Material("Cu"), P["E0"], P["Emin"], P["s_tilt"], N, seed=SEED, mode="cont", bethe="JL")
    return g.tally, c


def oracle_hists(c):
    bks = c["outcome"] == 1
    hE = binned(c["final_E"][bks], 100.0, 200)
    theta = np.degrees(np.arccos(np.clip(-c["dir"][bks, 2], -1.0, 1.0)))
    hT = binned(theta, 1.0, 90)
    return hE, hT


def homogeneous(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    keep = (a + b) > 0
    return stats.chi2_contingency(np.vstack([a[keep], b[keep]]))[1]


def test_yield_and_histograms_match_oracle(runs):
    t, c = runs
    n_bks = int((c["outcome"] == 1).sum())
    assert t["bks"] + t["abs"] + t["trsm"] + t["long"] == N
    assert eta_z(N, t["bks"], N, n_bks) < 3.0
    hE, hT = oracle_hists(c)
    gE = np.asarray(t["hist_E"][:200])
    gT = np.asarray(t["hist_T"][:90])
    assert abs(int(gE.sum()) - int(hE.sum())) <= 3 + 1e-3 * hE.sum()
    assert homogeneous(gE, hE) > 1e-3
    assert homogeneous(gT, hT) > 1e-3
    # the same electrons on the same stream: FP32 moves few of them
    assert np.abs(gE.astype(np.int64) - hE).sum() <= 0.05 * hE.sum()


def test_batched_equals_plain_histograms(runs):
    t, _ = runs
    b = engine.Batch([dict(P, num_el=N)], seed=SEED)
    res, status = b.run(_lib.Tune(1024, 0, 1, 0, 0))
    assert status == 0
    r = res[0]
    for k in ("bks", "abs", "trsm", "long", "events"):
        assert r[k] == t[k], k
    assert np.array_equal(r["hist_E"], t["hist_E"])
    assert np.array_equal(r["hist_T"], t["hist_T"])
