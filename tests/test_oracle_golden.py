"""The oracle against the reference's own outputs (tests/golden, generated by
tests/golden/gen_golden.py from the reference itself), and the C oracle
against the Python oracle.  CPU only."""
import math

import numpy as np
import pytest

import coracle
import mcd_oracle as O


def rel(a, b):
    a = np.asarray(a, dtype=float)
    b = np.asarray(b, dtype=float)
    m = np.isfinite(b)
    assert np.array_equal(np.isfinite(a), m)
    if not m.any():
        return 0.0
    return float(np.max(np.abs(a[m] - b[m]) / np.maximum(np.abs(b[m]), 1e-300)))


@pytest.mark.parametrize("sp", list(O.SPECIES))
def test_physics_functions(golden, sp):
    P = golden["physics"]
    E = P["E"]
    mat = O.Material(sp)
    assert rel([mat.atnd, mat.plasmon_e, mat.fermi_e], P[sp + "/const"]) < 1e-14
    assert rel([O.alpha(e, mat.Z) for e in E], P[sp + "/alpha"]) < 1e-14
    assert rel([O.ruther_sigma(e, mat.Z) for e in E], P[sp + "/ruth"]) < 1e-14
    assert rel([O.ruther_sigma_wDefl(e, mat.Z) for e in E], P[sp + "/ruth_wdefl"]) < 1e-14
    assert rel([O.ruther_N_sigma(e, mat.Z) for e in E], P[sp + "/ruth_nigram"]) < 1e-14
    assert rel([O.ruther_N_sigma_wDefl(e, mat.Z) for e in E], P[sp + "/ruth_nigram_wdefl"]) < 1e-14
    if sp + "/xip_g" in P:
        assert mat.xip_g == float(P[sp + "/xip_g"])
        assert rel([O.diffr_sigma(mat.xip_g, mat.atnd)], [float(P[sp + "/diffr"])]) < 1e-14
    else:
        assert mat.xip_g is None
    for Wc in (10.0, 50.0, 100.0):
        assert rel([O.moller_sigma(e, Wc, mat.n_val) for e in E], P[sp + "/moller/%g" % Wc]) < 1e-14
    for name, Es, ns in mat.shells:
        assert rel([O.gryz_sigma(e, Es, ns) for e in E], P[sp + "/gryz/" + name]) < 1e-14
    # Quinn's sqrt(a) - sqrt(a - b) cancels: ulp differences of Ef grow to ~1e-13
    assert rel([O.quinn_sigma(e, mat.plasmon_e, mat.fermi_e, mat.atnd) for e in P[sp + "/quinn_E"]],
               P[sp + "/quinn"]) < 1e-12
    Eb = P[sp + "/bethe_E"]
    for model, key in (("classical", "bethe_cl"), ("JL", "bethe_jl"), ("explicit", "bethe_ex")):
        assert rel([O.stopping_power(model, mat, e) for e in Eb], P[sp + "/" + key]) < 1e-14
    EE, WW = P[sp + "/dcs_E"], P[sp + "/dcs_W"]
    assert rel(O.moller_dcs(EE, WW, mat.n_val), P[sp + "/moller_dcs"]) < 1e-14
    _, Eb_, ns_ = mat.outer_shell
    assert rel(O.gryz_dcs(EE, WW, ns_, Eb_), P[sp + "/gryz_dcs"]) < 1e-14
    bc = [[O.binary_coll_c2(e, w, mat.fermi_e) for w in P[sp + "/bc_W"]] for e in EE[:, 0]]
    assert rel(bc, P[sp + "/bc"]) < 1e-15       # NaN pattern checked inside rel
    assert rel([O.rutherford_c2(e, mat.Z, u) for e, u in P[sp + "/ruth_EU"]], P[sp + "/ruth_c2"]) < 1e-14
    assert rel([O.maxW(e, mat.fermi_e) for e in EE[:, 0]], P[sp + "/maxW"]) < 1e-15


def test_detector_projection_matches_reference(golden):
    """rotation.py:78-102 at the geometry of parameters.py:22-33 and at other
    tilts, on seeded unit directions and the six axis directions."""
    P = golden["physics"]
    for a in P["det/alphas"]:
        got = O.proj_on_detector(P["det/dirs"], a, P["det/xy_PC"], float(P["det/L"]))
        assert np.max(np.abs(got - P["det/xy/%g" % a])) <= 1e-12 * 6000.0, a


def test_table_cdf_matches_reference(golden):
    """Every table the benchmarks sample: unmasked counts exact, values within
    one float32 step of the reference's table (the reference evaluates parts
    of dsigma/dW in float32)."""
    T = golden["tables"]
    for key in T["names"]:
        sp = str(T[key + "/species"])
        kind = key.split("/")[1]
        mat = O.Material(sp)
        cdf, valid = O.table_cdf(kind, mat, T[key + "/Ws"], T[key + "/Es"])
        s32 = O.table_store32(cdf, valid)
        assert np.array_equal((s32 != 0).sum(axis=1), T[key + "/nvalid"]), key
        rows = T[key + "/rows"]
        d = np.abs(s32[rows].astype(np.float64) - T[key + "/cdf_rows"].astype(np.float64))
        assert d.max() <= 2.0 ** -24 + 1e-12, key
        rs = np.abs(s32.astype(np.float64).sum(axis=1) - T[key + "/rowsum"])
        assert rs.max() < 1e-5, key
        tol = float(T[key + "/spec"][3])
        assert d.max() < tol


def _tables_for(T, name, mat):
    out = []
    for kind in ("Moller", "Gryz"):
        key = name + "/" + kind
        cdf, valid = O.table_cdf(kind, mat, T[key + "/Ws"], T[key + "/Es"])
        out.append(O.Table(T[key + "/Ws"], T[key + "/Es"], O.table_store32(cdf, valid)))
    return out


REPLAYS = [("ds_si", "cfg1"), ("ds_au", "cfg3"), ("cont_al", None), ("cont_cu", None),
           ("ds_si_nigram", "cfg1"), ("ds_si_nigram_wdefl", "cfg1"), ("ds_si_diff", "cfg1"),
           ("cont_al_nigram", None)]


@pytest.mark.parametrize("tag,tname", REPLAYS)
def test_replay_reference_trajectories(golden, tag, tname):
    """Whole trajectories of the reference, replayed on its own MT19937 stream:
    same channel sequence, same outcome rows, values within 1e-9.  Besides the
    default model: Nigram elastic cross sections (DS and continuous), and the
    diffraction channel of diffMFP in a 3000 A Si film, run by the reference
    with its extinction distance supplied (its constructor reads self.xip_g,
    whose assignment is commented out)."""
    R = golden["replay"]
    mat = O.Material(str(R[tag + "/species"]))
    cfg = R[tag + "/cfg"]
    evo, rwo = R[tag + "/ev_off"], R[tag + "/row_off"]
    tabs = _tables_for(golden["tables"], tname, mat) if tname else None
    elastic = str(R[tag + "/elastic"]) if tag + "/elastic" in R else "Ruth_vanilla"
    diff = bool(R[tag + "/diffMFP"]) if tag + "/diffMFP" in R else False
    maxz = float(R[tag + "/thickness"]) if tag + "/thickness" in R else 1e30
    for k, seed in enumerate(R[tag + "/seeds"]):
        el = O.Electron(cfg[0], cfg[1], O.beam_direction(cfg[2]), record=True)
        if tag.startswith("ds"):
            O.trajectory_ds(el, mat, cfg[3], 10 ** 9, maxz, tabs, O.MTStream(int(seed)), elastic, diff)
        else:
            O.trajectory_cont(el, mat, 10 ** 9, maxz, "classical", O.MTStream(int(seed)), elastic=elastic)
        a, b = evo[k], evo[k + 1]
        assert len(el.events) == b - a
        ev = np.array(el.events, dtype=float)
        cols = [("E_loss", 2), ("pol_angle", 3), ("az_angle", 4), ("pathl", 5), ("energy", 9)]
        if tag.startswith("ds"):
            types = R[tag + "/ev/type"][a:b].copy()
            types[types == 3 + len(mat.shells)] = O.CH_DIFF     # the label list ends with 'diff'
            assert np.array_equal(ev[:, 0].astype(int), types)
            cols += [("E", 1), ("x", 6), ("y", 7), ("z", 8)]
        for col, ci in cols:
            ref = R[tag + "/ev/" + col][a:b]
            scale = 1e4 if col in ("x", "y", "z") else 1.0
            d = np.abs(ev[:, ci] - ref)
            m = np.isfinite(ref)
            assert np.array_equal(np.isnan(ev[:, ci]), np.isnan(ref))
            assert np.all(d[m] <= 1e-9 * np.maximum(np.abs(ref[m]), scale)), (tag, k, col)
        ra, rb = rwo[k], rwo[k + 1]
        assert [r[0] for r in el.rows] == list(R[tag + "/row/outcome"][ra:rb])
        for i, (_, fe, d, p) in enumerate(el.rows):
            assert abs(fe - R[tag + "/row/final_E"][ra + i]) <= 1e-9 * fe
            assert np.allclose(d, [R[tag + "/row/" + c][ra + i] for c in ("dx", "dy", "dz")], rtol=0, atol=1e-9)
            assert np.allclose(p, [R[tag + "/row/" + c][ra + i] for c in ("last_x", "last_y", "last_z")],
                               rtol=1e-9, atol=1e-6)


def test_diffraction_replay_reaches_trdf(golden):
    """The diffraction fixture exercises the channel and the 'trdf' exit."""
    R = golden["replay"]
    assert (R["ds_si_diff/ev/type"] == 6).sum() >= 3
    assert (R["ds_si_diff/row/outcome"] == "trdf").sum() >= 1


def test_abs_row_keeps_pre_loss_energy(golden):
    """MC/tools/electron.py:48-56: saveOutcomes runs before the energy is
    updated, so an 'abs' row holds the energy before the last loss (> Emin)."""
    R = golden["replay"]
    oc = R["ds_si/row/outcome"]
    fe = R["ds_si/row/final_E"]
    Emin = R["ds_si/cfg"][1]
    assert (oc == "abs").any()
    assert np.all(fe[oc == "abs"] > Emin)


PHILOX_KAT = [
    # Random123 known-answer vectors for philox4x32-10: (ctr, key, out)
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF, 0xFFFFFFFF), (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]


@pytest.mark.parametrize("ctr,key,out", PHILOX_KAT)
def test_philox_known_answers(ctr, key, out):
    assert O.philox4x32_10(ctr, key) == out


def test_c_oracle_equals_python_oracle(golden):
    """The C twin (used for large samples and the CPU baseline) reproduces the
    Python oracle bit for bit on the Philox stream."""
    T = golden["tables"]
    mat = O.Material("Si")
    hts = [coracle.HostTable.build(k, mat, T["cfg1/" + k + "/Ws"], T["cfg1/" + k + "/Es"]) for k in ("Moller", "Gryz")]
    pts = [O.Table(t.Ws, t.Es, t.cdf) for t in hts]
    n = 16
    c = coracle.run(mat, 10000.0, 1000.0, 0.0, n, seed=5, mode="DS", Wc=100.0, tables=hts, nthreads=3)
    py = O.run_ds(mat, 10000.0, 1000.0, 0.0, 100.0, 10 ** 15, 1e30, pts, n, 5)
    assert np.array_equal([O.OUT_CODE[e.rows[0][0]] for e in py], c["outcome"])
    assert np.array_equal([e.rows[0][1] for e in py], c["final_E"])
    assert np.array_equal([e.rows[0][2] for e in py], c["dir"])
    assert np.array_equal([e.rows[0][3] for e in py], c["last_pos"])
    assert np.array_equal([e.steps for e in py], c["n_events"])
    # elastic variants and the diffraction channel in a Si film
    for elastic, diff, th in (("Ruth_nigram", False, 1e30), ("Ruth_nigram_wDefl", False, 1e30),
                              ("Ruth_vanilla_wDefl", False, 1e30), ("Ruth_vanilla", True, 3000.0)):
        c = coracle.run(mat, 10000.0, 1000.0, 0.0, n, seed=5, mode="DS", Wc=100.0, tables=hts, nthreads=3,
                        elastic=elastic, diff=diff, thickness=th)
        py = O.run_ds(mat, 10000.0, 1000.0, 0.0, 100.0, 10 ** 15, th, pts, n, 5, elastic=elastic, diff=diff)
        assert np.array_equal([O.OUT_CODE[e.rows[0][0]] for e in py], c["outcome"]), elastic
        assert np.array_equal([e.rows[0][1] for e in py], c["final_E"]), elastic
        assert np.array_equal([e.rows[0][2] for e in py], c["dir"]), elastic
        assert np.array_equal([e.steps for e in py], c["n_events"]), elastic
    m2 = O.Material("Al")
    c = coracle.run(m2, 15000.0, 1000.0, 70.0, 8, seed=9, mode="cont", nthreads=2, elastic="Ruth_nigram")
    py = O.run_cont(m2, 15000.0, 1000.0, 70.0, 10 ** 15, 1e30, "classical", 8, 9, elastic="Ruth_nigram")
    assert np.array_equal([e.rows[0][1] for e in py], c["final_E"])
    for model in ("classical", "JL", "explicit"):
        m2 = O.Material("Cu")
        c = coracle.run(m2, 20000.0, 1000.0, 70.0, 8, seed=9, mode="cont", bethe=model, nthreads=2)
        py = O.run_cont(m2, 20000.0, 1000.0, 70.0, 10 ** 15, 1e30, model, 8, 9)
        assert np.array_equal([e.rows[0][1] for e in py], c["final_E"])
        assert np.array_equal([e.rows[0][2] for e in py], c["dir"])


def _eta_z(n1, k1, n2, k2):
    p = (k1 + k2) / (n1 + n2)
    s = math.sqrt(p * (1 - p) * (1.0 / n1 + 1.0 / n2))
    return abs(k1 / n1 - k2 / n2) / s


@pytest.mark.parametrize("tag,tname", [("si10", "cfg1"), ("al5", "cfg4_Al_5"), ("cu20t45", "cfg4_Cu_20")])
def test_c_oracle_statistics_match_reference(golden, tag, tname):
    """The oracle on its Philox stream against the reference's own large
    samples: eta within 3 sigma, exit energies and step counts by KS."""
    from scipy import stats
    S = golden["ref_stats"]
    T = golden["tables"]
    E0, Emin, tilt, Wc, _ = S[tag + "/cfg"]
    mat = O.Material(str(S[tag + "/species"]))
    hts = [coracle.HostTable.build(k, mat, T[tname + "/" + k + "/Ws"], T[tname + "/" + k + "/Es"])
           for k in ("Moller", "Gryz")]
    n = 8000
    c = coracle.run(mat, E0, Emin, tilt, n, seed=11, mode="DS", Wc=Wc, tables=hts)
    ref_oc = S[tag + "/outcome"]
    z = _eta_z(len(ref_oc), int((ref_oc == 1).sum()), n, int((c["outcome"] == 1).sum()))
    assert z < 3.0, z
    rb = S[tag + "/final_E"][ref_oc == 1]
    cb = c["final_E"][c["outcome"] == 1]
    assert stats.ks_2samp(rb, cb).pvalue > 0.01
    assert stats.ks_2samp(S[tag + "/nsteps"], c["n_events"]).pvalue > 0.01
