"""FP32 CUDA transport against the reference's own large samples
(tests/golden/ref_stats.npz, produced by running the reference): the same
kinds of statistical checks as the reference's tests/testThings.py (channel
mix at E0 by chi^2, polar and azimuthal angles, per-channel energy losses),
plus backscatter coefficient eta within 3 sigma and KS tests on exit
energies, exit angles, event counts and maximum depth, all at p > 0.01.

Every check runs on each FP32 code path: the plain launch with cross
sections evaluated per event, the plain launch reading its cross-section
table, and the persistent batched kernel in the configuration the benchmark
times (tabulated cross sections, two blocks of 576 per SM at 56 registers,
refill 1)."""
import numpy as np
import pytest
from scipy import stats

from mcd import _lib
from _gpu_util import VARIANTS, eta_z, input_par, run_variant, theta_deg

pytestmark = pytest.mark.gpu

STATS = {
    "si10": input_par("Si", 10000.0, 1000.0, 0.0),
    "au30": input_par("Au", 30000.0, 500.0, 70.0, Wc=50.0, tol=1e-4),
    "cu20t45": input_par("Cu", 20000.0, 1000.0, 45.0),
    "al5": input_par("Al", 5000.0, 1000.0, 0.0),
}
P_MIN = 0.01


@pytest.fixture(scope="module")
def runs():
    cache = {}

    def get(variant, tag):
        if (variant, tag) not in cache:
            n = 100000 if tag != "au30" else 20000
            cache[(variant, tag)] = run_variant(variant, STATS[tag], n, seed=2024)
        return cache[(variant, tag)]
    return get


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("tag", list(STATS))
def test_eta_and_exit_distributions(golden, runs, tag, variant):
    S = golden["ref_stats"]
    g = runs(variant, tag)
    e = g.electrons
    n = e["outcome"].size
    ro = S[tag + "/outcome"]
    z = eta_z(ro.size, int((ro == 1).sum()), n, int((e["outcome"] == 1).sum()))
    assert z < 3.0, (tag, z, g.eta, float((ro == 1).mean()))
    bks = e["outcome"] == 1
    rb = ro == 1
    assert stats.ks_2samp(S[tag + "/final_E"][rb], e["final_E"][bks]).pvalue > P_MIN
    th_ref = np.degrees(np.arccos(-S[tag + "/dir"][rb, 2]))
    th = np.degrees(np.arccos(np.clip(-e["dir"][bks, 2], -1, 1)))
    assert stats.ks_2samp(th_ref, th).pvalue > P_MIN
    assert stats.ks_2samp(S[tag + "/nsteps"], e["n_events"]).pvalue > P_MIN
    assert stats.ks_2samp(S[tag + "/zmax"], e["max_z"]).pvalue > P_MIN
    # the double-row rate ('bks' then 'abs' in one step)
    rate_ref = float((S[tag + "/nrows"] > 1).mean())
    rate = float((e["flags"] & 1).astype(bool).mean())
    assert abs(rate - rate_ref) < 3 * np.sqrt(max(rate_ref, 1e-4) * (1.0 / ro.size + 1.0 / n)) + 1e-4


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("tag", ["si10", "cu20t45", "al5"])
def test_first_event_channels_and_angles(golden, tag, variant):
    """Events at E0 (the first event of each electron): channel mix by chi^2,
    Rutherford polar angle and Moller energy loss by KS, azimuth uniform."""
    S = golden["ref_stats"]
    p = STATS[tag]
    n = 20000
    g = run_variant(variant, p, n, seed=99, electrons=False, ring_capacity=n * 1200)
    assert not (g.status & _lib.FLAG_RING_FULL)
    ev = g.events
    first = ev[(ev["step_chan"] >> 5) == 0]
    assert first.size == n
    ch = (first["step_chan"] & 31).astype(int)
    ref_first = S[tag + "/first"]
    ref_ch = ref_first[:, 0].astype(int)
    k = int(max(ch.max(), ref_ch.max())) + 1
    obs = np.bincount(ch, minlength=k)
    ref = np.bincount(ref_ch, minlength=k)
    keep = (obs + ref) > 0
    table = np.vstack([obs[keep], ref[keep]])
    assert stats.chi2_contingency(table)[1] > P_MIN
    # Rutherford polar angle at E0 (reference TestPolarProb_Ruth_E0)
    ru = theta_deg(first["c2"][ch == 0])
    ru_ref = theta_deg(ref_first[ref_ch == 0, 1])
    assert stats.ks_2samp(ru, ru_ref).pvalue > P_MIN
    # Moller energy loss at E0 (the W behind TestPolarProb_Moller_E0)
    mo = first["W"][ch == 1]
    mo_ref = ref_first[ref_ch == 1, 2]
    if mo_ref.size > 30:
        assert stats.ks_2samp(mo, mo_ref).pvalue > P_MIN
    # azimuth 2*halfPhi uniform on [0, 2pi) (reference TestAzimProb_Ruth);
    # every 97th event in (electron, event) order, not in the ring's order
    ev = ev[np.lexsort(((ev["step_chan"] >> 5), ev["electron"]))]
    phi = 2.0 * ev["half_phi"][::97].astype(np.float64)
    assert stats.kstest(phi / (2 * np.pi), "uniform").pvalue > P_MIN


@pytest.mark.parametrize("variant", VARIANTS)
@pytest.mark.parametrize("tag", ["si10", "cu20t45"])
def test_all_energy_samples(golden, tag, variant):
    """Every-128th event of the reference against every-128th event here:
    Rutherford polar angle and inelastic energy losses over all energies
    (reference TestPolarProb_Ruth / TestPolarProb_Moller)."""
    S = golden["ref_stats"]
    p = STATS[tag]
    n = 16000
    g = run_variant(variant, p, n, seed=5, electrons=False, ring_capacity=n * 1200)
    assert not (g.status & _lib.FLAG_RING_FULL)
    ev = g.events
    ev = ev[np.lexsort(((ev["step_chan"] >> 5), ev["electron"]))]
    steps = ev["step_chan"] >> 5
    ev = ev[steps % 128 == 0]
    ch = (ev["step_chan"] & 31).astype(int)
    sm = S[tag + "/sample"]
    rch = sm[:, 0].astype(int)
    assert stats.ks_2samp(theta_deg(ev["c2"][ch == 0]), theta_deg(sm[rch == 0, 3])).pvalue > P_MIN
    assert stats.ks_2samp(ev["E"], sm[:, 1]).pvalue > P_MIN
    for c in (1, 3 + {"si10": 2, "cu20t45": 3}[tag]):
        a, b = ev["W"][ch == c], sm[rch == c, 2]
        if min(a.size, b.size) > 30:
            assert stats.ks_2samp(a, b).pvalue > P_MIN, c
