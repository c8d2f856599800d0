"""CUDA transport against the oracle on the same inputs.

FP64 transport and the C oracle consume the same Philox stream and the same
tables, so they follow the same trajectories: outcome, event count and exit
energy agree electron by electron (a trajectory can still part where CUDA's
log/sin and glibc's differ in the last bit right at a decision boundary,
hence the 99% floor).  FP32 transport is checked against the oracle
statistically and by its per-electron agreement rate.
"""
import math

import mcd_oracle as O
import numpy as np
import pytest
import torch
from scipy import stats

from mcd import _lib, engine, tables
from _gpu_util import eta_z, input_par, run_pair

pytestmark = pytest.mark.gpu

CASES = [
    # name, input parameters, electrons
    ("si10_ds", input_par("Si", 10000.0, 1000.0, 0.0), 3000),
    ("cu20t45_ds", input_par("Cu", 20000.0, 1000.0, 45.0), 600),
    ("au30t70_ds", input_par("Au", 30000.0, 500.0, 70.0, Wc=50.0, tol=1e-4), 200),
    ("al15_cont_cl", input_par("Al", 15000.0, 1000.0, 70.0, mode="cont", bethe="classical"), 3000),
    ("cu20_cont_jl", input_par("Cu", 20000.0, 1000.0, 70.0, mode="cont", bethe="JL"), 2000),
    ("si10_cont_ex", input_par("Si", 10000.0, 1000.0, 0.0, mode="cont", bethe="explicit"), 2000),
    # elastic models (MC/tools/crossSections.py:63-147) and the diffraction
    # channel in a 3000 A Si film (diffMFP, 'trdf' exits)
    ("si10_ds_nigram", input_par("Si", 10000.0, 1000.0, 0.0, elastic="Ruth_nigram"), 2000),
    ("cu20_ds_nigram_wdefl", input_par("Cu", 20000.0, 1000.0, 45.0, elastic="Ruth_nigram_wDefl"), 400),
    ("si_film_diff", input_par("Si", 10000.0, 1000.0, 0.0, diffMFP=True, thickness=3000.0), 3000),
    ("al15_cont_nigram", input_par("Al", 15000.0, 1000.0, 70.0, mode="cont", elastic="Ruth_nigram"), 2000),
]


@pytest.mark.parametrize("name,p,n", CASES, ids=[c[0] for c in CASES])
def test_fp64_follows_oracle_trajectories(name, p, n):
    g, c = run_pair(p, n, seed=123, precision="fp64")
    e = g.electrons
    same = (e["outcome"] == c["outcome"]) & (e["n_events"] == c["n_events"])
    assert same.mean() >= 0.99, (name, same.mean())
    fe_ok = np.abs(e["final_E"] - c["final_E"]) <= 1e-9 * np.abs(c["final_E"])
    assert (same & fe_ok).mean() >= 0.99, name
    d_ok = np.abs(e["dir"] - c["dir"]).max(axis=1) <= 1e-9
    d_ok |= np.isnan(c["dir"]).any(axis=1) & np.isnan(e["dir"]).any(axis=1)
    assert (same & d_ok).mean() >= 0.99, name
    p_ok = np.abs(e["last_pos"] - c["last_pos"]).max(axis=1) <= 1e-9 * np.maximum(1.0, np.abs(c["last_pos"]).max(axis=1))
    assert (same & p_ok).mean() >= 0.98, name
    # tallies agree with the per-electron rows
    t = g.tally
    assert t["bks"] == int((e["outcome"] == 1).sum())
    assert t["events"] == int(e["n_events"].sum())
    assert t["bks"] + t["abs"] + t["trsm"] + t["trdf"] + t["long"] == n
    if p.get("diffMFP"):
        assert t["trdf"] == int((e["outcome"] == 4).sum()) > 0
        assert abs(t["trdf"] - int((c["outcome"] == 4).sum())) <= 0.01 * n


DS_CASES = [c for c in CASES if "_ds" in c[0] or c[0] == "si_film_diff"]


@pytest.mark.parametrize("name,p,n", DS_CASES, ids=[c[0] for c in DS_CASES])
def test_fp64_tabulated_follows_oracle_trajectories(name, p, n):
    """FP64 transport reading its FP64 cross-section table (cubics on
    octave grids, within about 1.3e-10 of the exact values; exact where a
    channel threshold lies in the cell) follows the oracle like the inline
    path: a channel decision moves only when a draw falls that close to a
    boundary."""
    g, c = run_pair(p, n, seed=123, precision="fp64", tabulated=True)
    e = g.electrons
    same = (e["outcome"] == c["outcome"]) & (e["n_events"] == c["n_events"])
    assert same.mean() >= 0.99, (name, same.mean())
    fe_ok = np.abs(e["final_E"] - c["final_E"]) <= 1e-9 * np.abs(c["final_E"])
    assert (same & fe_ok).mean() >= 0.99, name
    d_ok = np.abs(e["dir"] - c["dir"]).max(axis=1) <= 1e-9
    d_ok |= np.isnan(c["dir"]).any(axis=1) & np.isnan(e["dir"]).any(axis=1)
    assert (same & d_ok).mean() >= 0.99, name
    assert g.tally["bks"] + g.tally["abs"] + g.tally["trsm"] + g.tally["trdf"] + g.tally["long"] == n


SIG64_CASES = [("Si", 100.0, 100.0), ("Al", 100.0, 100.0), ("Cu", 100.0, 100.0), ("Au", 100.0, 50.0)]


@pytest.mark.parametrize("sp,Emin,Wc", SIG64_CASES, ids=[c[0] for c in SIG64_CASES])
def test_fp64_sigma_table_against_the_oracle_cross_sections(sp, Emin, Wc):
    """The FP64 table mcd_build_sigma_table writes, read back and evaluated
    on the host as the transport reads it (octave from the exponent, cell
    and offset from the mantissa, Horner in each column), against the
    oracle's cross sections at 3000 seeded energies over (Emin, 30 keV]: the
    mean free path within 3e-10 relative and the running-sum fractions
    within 3e-10 absolute in every unflagged cell, and a cell is flagged
    exactly when a channel threshold lies in the span of its four nodes or
    its lowest node lies below 2 Wc (the Moller cross section is negative
    there, with a pole at Wc)."""
    p = input_par(sp, 30000.0, Emin, 0.0, Wc=Wc)
    mat = _lib.material(sp)
    sim = engine.make_sim(p, 16, precision=_lib.FP64)
    assert tables.sigma_table_fits(sim, mat)
    tab = tables.sigma_table(sim, mat).view(torch.float64).cpu().numpy()
    om = O.Material(sp)
    K = 3 + len(om.shells)
    stride = tables.sig64_stride(K)
    e_lo = math.frexp(Emin)[1] - 1
    thresholds = [Wc, om.plasmon_e] + [Es for _, Es, _ in om.shells]
    rng = np.random.default_rng(11)
    worst_mfp, worst_frac, flagged = 0.0, 0.0, 0
    for E in np.exp(rng.uniform(math.log(Emin), math.log(30000.0), 3000)):
        m, ex = math.frexp(E)          # E = m 2^ex, m in [0.5, 1)
        t = (2.0 * m - 1.0) * tables.SIG64_CELLS
        i = int(t)
        f = t - i
        rec = tab[((ex - 1 - e_lo) * tables.SIG64_CELLS + i) * stride:][:stride]
        h = 2.0 ** (ex - 1) / tables.SIG64_CELLS
        E1 = 2.0 ** (ex - 1) + (i - 1) * h
        kink = any(E1 <= x <= E1 + 3 * h for x in thresholds) or E1 < 2 * Wc
        assert (rec[0] != 0.0) == kink, (sp, E)
        if kink:
            flagged += 1
            continue
        c = rec[2:].reshape(K, 4)
        val = ((c[:, 3] * f + c[:, 2]) * f + c[:, 1]) * f + c[:, 0]
        sig = [v for _, v in O.ds_sigmas(E, om, Wc)]
        tot = sum(sig)
        worst_mfp = max(worst_mfp, abs(val[0] / O.mfp_from_sigma(tot, om.atnd) - 1.0))
        worst_frac = max(worst_frac, float(np.max(np.abs(val[1:] - np.cumsum(sig)[:-1] / tot))))
    assert worst_mfp < 3e-10 and worst_frac < 3e-10, (sp, worst_mfp, worst_frac)
    assert flagged < 450     # 100-200 eV (below 2 Wc) is about 12% of the log-uniform energies


def test_fp64_table_on_a_range_bounded_by_powers_of_two():
    """E0 = 8192 eV starts an octave block of its own and Emin = 1024 eV ends
    the lowest one: the FP64 table still follows the oracle."""
    p = input_par("Al", 8192.0, 1024.0, 20.0)
    g, c = run_pair(p, 1500, seed=77, precision="fp64", tabulated=True)
    e = g.electrons
    same = (e["outcome"] == c["outcome"]) & (e["n_events"] == c["n_events"])
    assert same.mean() >= 0.99, same.mean()
    fe_ok = np.abs(e["final_E"] - c["final_E"]) <= 1e-9 * np.abs(c["final_E"])
    assert (same & fe_ok).mean() >= 0.99


@pytest.mark.parametrize("tabulated", [True, False], ids=["table", "inline"])
@pytest.mark.parametrize("name", ["si10_ds", "si_film_diff"])
def test_fp64_small_run_kernel_equals_plain(name, tabulated):
    """A small FP64 DS run on the automatic block size goes to the kernel
    whose idle half-warp lanes compute each event's Philox block, step
    logarithm and azimuth ahead; its rows and tallies equal the plain
    kernel's (two threads per block) bit for bit."""
    p = next(c[1] for c in CASES if c[0] == name)
    a = engine.run(p, num_el=1000, seed=31, precision="fp64", tabulated=tabulated, block_size=0)
    b = engine.run(p, num_el=1000, seed=31, precision="fp64", tabulated=tabulated, block_size=2)
    for k in ("outcome", "n_events", "flags"):
        assert np.array_equal(a.electrons[k], b.electrons[k]), k
    for k in ("final_E", "dir", "last_pos", "max_z"):      # NaN directions (the reference's quirk) included
        assert np.array_equal(a.electrons[k], b.electrons[k], equal_nan=True), k
    for k in ("bks", "abs", "trsm", "trdf", "long", "events", "double_rows"):
        assert a.tally[k] == b.tally[k], k


def test_fp64_table_equals_inline_on_the_small_configuration():
    """The small FP64 configuration (Si 10 keV, 1000 electrons): with the
    table every trajectory matches the inline run's."""
    p = input_par("Si", 10000.0, 1000.0, 0.0)
    a = engine.run(p, num_el=1000, seed=0, precision="fp64")
    b = engine.run(p, num_el=1000, seed=0, precision="fp64", tabulated=True)
    ea, eb = a.electrons, b.electrons
    same = (ea["outcome"] == eb["outcome"]) & (ea["n_events"] == eb["n_events"])
    assert same.mean() >= 0.999, same.mean()
    assert np.all(np.abs(ea["final_E"][same] - eb["final_E"][same]) <= 1e-9 * np.abs(ea["final_E"][same]))


@pytest.mark.parametrize("name,p,n", CASES, ids=[c[0] for c in CASES])
def test_fp32_matches_oracle_statistics(name, p, n):
    n = n * 4
    g, c = run_pair(p, n, seed=7, precision="fp32")
    e = g.electrons
    agree = np.mean((e["outcome"] == c["outcome"]) & (e["n_events"] == c["n_events"]))
    assert agree > 0.5, agree      # same stream: most trajectories stay identical in FP32
    k1 = int((e["outcome"] == 1).sum())
    k2 = int((c["outcome"] == 1).sum())
    assert eta_z(n, k1, n, k2) < 3.0
    b1 = e["final_E"][e["outcome"] == 1]
    b2 = c["final_E"][c["outcome"] == 1]
    if min(b1.size, b2.size) > 20:
        assert stats.ks_2samp(b1, b2).pvalue > 0.01
    assert stats.ks_2samp(e["n_events"], c["n_events"]).pvalue > 0.01
    # FP32 error against the FP64 oracle on the electrons that stayed identical
    same = (e["outcome"] == c["outcome"]) & (e["n_events"] == c["n_events"])
    relE = np.abs(e["final_E"][same] - c["final_E"][same]) / c["final_E"][same]
    # FP32 subtraction rounding over a few hundred losses: ~1e-5 relative
    assert np.median(relE) < 1e-4
