"""The theory-distribution tools of the oracle (CPU): the Watson U^2 of the
reference's tests (tests/testThings.py:255-316) and the integrated
energy-loss CDFs of MC/tools/distributions.py:21-124, which use
scipy.integrate.quad."""
import numpy as np
import pytest
from scipy import integrate

import mcd_oracle as O


def u2_loop(x, y):
    """The reference's loop, step by step: walk the sorted unique pooled
    values and record the empirical CDF difference at each."""
    x, y = sorted(x), sorted(y)
    nx, ny = len(x), len(y)
    N = nx + ny
    xi, yi, dk = [0], [0], []
    for v in sorted(set(x + y)):
        if v in x:
            xi.append(len(x) - x[::-1].index(v))     # count of x <= v
        if v in y:
            yi.append(len(y) - y[::-1].index(v))
        dk.append(xi[-1] / nx - yi[-1] / ny)
    dk = np.array(dk)
    return nx * ny * (np.sum(dk ** 2) - np.sum(dk) ** 2 / N) / N ** 2


def test_watson_u2_matches_loop_form():
    rng = np.random.default_rng(0)
    for _ in range(5):
        x = list(np.round(rng.uniform(0, 90, 60), 1))     # rounded: ties inside and across samples
        y = list(np.round(rng.uniform(0, 100, 45), 1))
        assert abs(O.watson_u2(x, y) - u2_loop(x, y)) < 1e-12


def test_watson_u2_pvalue_points():
    # the reference's critical value 0.152 is the 10% point
    assert abs(O.watson_u2_pvalue(0.152) - 0.10) < 2e-3
    assert abs(O.watson_u2_pvalue(0.187) - 0.05) < 2e-3
    assert O.watson_u2_pvalue(0.0) == 1.0


@pytest.mark.parametrize("kind,E", [("Moller", 20000.0), ("Moller", 16000.0), ("Gryz", 20000.0)])
def test_theory_W_cdf_matches_quad(kind, E):
    mat = O.Material("Al")
    wmin = 10.0 if kind == "Moller" else mat.outer_shell[1]
    W, c = O.theory_W_cdf(kind, mat, E, wmin)
    if kind == "Moller":
        f = lambda w: float(O.moller_dcs(E, w, mat.n_val))
    else:
        _, Eb, ns = mat.outer_shell
        f = lambda w: float(O.gryz_dcs(E, w, ns, Eb))
    wmax = O.maxW(E, mat.fermi_e)
    tot = integrate.quad(f, wmin, wmax, epsabs=0, limit=200, points=[wmin * 2, wmin * 10])[0]
    for q in (wmin * 1.5, wmin * 5, wmin * 40, wmax * 0.5):
        ref = integrate.quad(f, wmin, q, epsabs=0, limit=200)[0] / tot
        got = np.interp(q, W, c)
        assert abs(got - ref) < 2e-5, (q, got, ref)
