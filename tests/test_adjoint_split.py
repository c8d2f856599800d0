"""The per-electron split of the re-simulated finite difference (host
arithmetic, on CPU tensors): its parts add up to the central difference of
the loss when the bins are the soft bins of the quantities, an electron whose
quantity and event are the same in both runs carries nothing, and the jump
part's standard error is the root sum of squares of the jumping terms."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
from mcd import adjoint  # noqa: E402

SIGMA, LO, HI, NB = 40.0, 1000.0, 5000.0, 32
CB = LO + (np.arange(NB) + 0.5) * (HI - LO) / NB


def soft_bins(q, k, n):
    w = np.exp(-(q[:, None] - CB[None, :]) ** 2 / (2 * SIGMA * SIGMA))
    return (w * (k >= 0)[:, None]).sum(0) / n


def pair(n=5000, seed=1, h=1e-3):
    rng = np.random.default_rng(seed)
    qm = rng.uniform(LO, HI, n)
    qp = qm + rng.normal(0.0, 5.0, n)                  # the smooth shift
    km = rng.integers(-1, 40, n)
    kp = km.copy()
    jump = rng.random(n) < 0.03                         # another event sequence
    kp[jump] = rng.integers(-1, 40, int(jump.sum()))
    qp[jump] = rng.uniform(LO, HI, int(jump.sum()))
    return qm, qp, km, kp, h


def split(qm, qp, km, kp, h, target):
    n = len(qm)
    hm, hp = soft_bins(qm, km, n), soft_bins(qp, kp, n)
    T = lambda a: torch.as_tensor(a)  # noqa: E731
    return adjoint.fd_split(T(qm), T(qp), T(km), T(kp), hm, hp, target, CB, SIGMA, h, n), hm, hp


def test_parts_add_up_to_the_difference():
    qm, qp, km, kp, h = pair()
    target = np.random.default_rng(2).uniform(0, 2e-3, NB)
    out, hm, hp = split(qm, qp, km, kp, h, target)
    want = (np.sum((hp - target) ** 2) - np.sum((hm - target) ** 2)) / (2 * h)
    assert out["fd"] == pytest.approx(want, rel=1e-12)
    assert out["fd_same_sequence"] + out["fd_jump"] == pytest.approx(out["fd"], rel=1e-9, abs=1e-15)
    assert out["changed"] == int((km != kp).sum())
    assert out["fd_jump"] != 0.0 and out["fd_same_sequence"] != 0.0


def test_unchanged_electrons_carry_nothing_and_jump_se():
    qm, qp, km, kp, h = pair(seed=3)
    same = km == kp
    qp[same] = qm[same]                                 # only the jumpers move
    target = np.zeros(NB)
    out, hm, hp = split(qm, qp, km, kp, h, target)
    assert out["fd_same_sequence"] == 0.0
    assert out["fd_jump"] == pytest.approx(out["fd"], rel=1e-9)
    # the jump terms by hand
    g = 2.0 * (0.5 * (hm + hp) - target)
    K = lambda q, k: np.exp(-(q[:, None] - CB[None, :]) ** 2 / (2 * SIGMA * SIGMA)) @ g * (k >= 0)  # noqa: E731
    ce = (K(qp, kp) - K(qm, km)) / (2 * h * len(qm))
    assert out["jump_se"] == pytest.approx(np.sqrt(np.sum(ce[~same] ** 2)), rel=1e-12)


def test_identical_runs_give_zero():
    qm, _, km, _, h = pair(seed=4)
    out, _, _ = split(qm, qm.copy(), km, km.copy(), h, np.full(NB, 1e-4))
    assert out["fd"] == 0.0 and out["fd_jump"] == 0.0 and out["fd_same_sequence"] == 0.0
    assert out["changed"] == 0 and out["jump_se"] == 0.0
