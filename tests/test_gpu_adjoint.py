"""Adjoint of the continuous-mode exit-energy tallies (mcd_adjoint).

Loss: L = sum_b (h_b(J, n) - t_b)^2 over 64 Gaussian-soft exit-energy bins
(sigma 50 eV), target t produced with J x 1.1 on the same random numbers.
The adjoint gives the pathwise derivative with the random numbers and the
event sequence frozen; it is checked against central finite differences of
exactly that function (the exit energies recomputed along the frozen event
sequence, mcd_adjoint_chain), in FP64 and in FP32, and against the FP64
adjoint.  The re-simulated finite difference (common random numbers, event
sequence free to change) is split into the electrons whose exit event
stayed the same and the jump part of those whose exit event changed."""
import numpy as np
import pytest
import torch

from mcd.adjoint import ExitEnergyModel, exit_histogram, resimulated_fd
from _gpu_util import input_par

pytestmark = pytest.mark.gpu

AL = input_par("Al", 15000.0, 1000.0, 70.0, mode="cont", bethe="classical")


def loss_grad(model, t):
    h, s, nb = model.forward(1.0, 1.0)
    L = float(np.sum((h - t) ** 2))
    dJ, dn = model.backward(2.0 * (h - t), 0.0)
    return L, dJ, dn


def chain_loss(model, t, J, n=1.0):
    h, _, _ = model.chain(J, n)
    return float(np.sum((h - t) ** 2))


@pytest.mark.parametrize("bethe", ["classical", "JL"])
def test_fp64_adjoint_equals_frozen_fd(bethe):
    p = dict(AL, Bethe_model=bethe)
    m = ExitEnergyModel(p, 20000, seed=11, precision="fp64")
    t, _, _ = m.forward(1.1, 1.0)
    L, dJ, dn = loss_grad(m, t)
    assert L > 0 and dJ != 0.0
    d = 1e-5
    fd = (chain_loss(m, t, 1 + d) - chain_loss(m, t, 1 - d)) / (2 * d)
    assert abs(dJ - fd) <= 1e-5 * abs(fd), (dJ, fd)
    # the exit energy does not depend on the density (s ~ 1/n, S ~ n)
    fdn = (chain_loss(m, t, 1.0, 1 + 1e-3) - chain_loss(m, t, 1.0, 1 - 1e-3)) / 2e-3
    assert abs(dn) <= 1e-9 * abs(dJ)
    assert abs(fdn) <= 1e-6 * abs(dJ)


def test_explicit_law_has_no_J_dependence():
    p = dict(AL, Bethe_model="explicit")
    m = ExitEnergyModel(p, 5000, seed=3, precision="fp64")
    t, _, _ = m.forward(1.0, 1.0)
    t = t * 0.9
    L, dJ, dn = loss_grad(m, t)
    assert dJ == 0.0


def test_fp32_adjoint_against_fd_and_fp64():
    m32 = ExitEnergyModel(AL, 50000, seed=5, precision="fp32")
    m64 = ExitEnergyModel(AL, 50000, seed=5, precision="fp64")
    t, _, _ = m64.forward(1.1, 1.0)
    _, dJ32, _ = loss_grad(m32, t)
    _, dJ64, _ = loss_grad(m64, t)
    d = 1e-3
    fd32 = (chain_loss(m32, t, 1 + d) - chain_loss(m32, t, 1 - d)) / (2 * d)
    assert abs(dJ32 - fd32) <= 1e-3 * abs(fd32), (dJ32, fd32)
    # FP32 transport against the FP64 forward: a few trajectories differ
    assert abs(dJ32 - dJ64) <= 2e-2 * abs(dJ64), (dJ32, dJ64)


def test_full_resimulation_fd_is_close():
    """The gradient check of the differentiable workload: a central finite
    difference at relative step 1e-3 with common random numbers, every
    electron re-simulated at J (1 +- 1e-3), at the workload's size (Al
    15 keV, 70 deg, 1e6 electrons, FP32).  Re-simulation lets about 0.35% of the
    electrons change their exit event; their soft-bin terms jump, so the
    difference is the pathwise derivative plus a jump part whose standard
    error (from its independent per-electron terms) is about 10% of the
    gradient at this size, shrinking as 1/sqrt(N h).  Over 16 seeds the jump
    part averaged 1.3% +- 2.9% of the gradient: no bias the pathwise
    estimator misses.  So the checks are
      * the electrons whose exit event stayed the same: their difference
        equals the adjoint within 2% (0.05-1.6% over 16 seeds; the rest is
        the pathwise terms of the electrons that changed, which this part
        leaves out, and it falls as 1/sqrt(N): 0.01-0.3% at 4e6);
      * the whole difference: within 4 standard errors of its jump part."""
    m = ExitEnergyModel(AL, 1000000, seed=7, precision="fp32")
    t, _, _ = m.forward(1.1, 1.0)
    _, dJ, _ = loss_grad(m, t)
    r = resimulated_fd(m, t, h=1e-3)
    assert np.sign(r["fd_same_sequence"]) == np.sign(dJ)
    assert abs(dJ - r["fd_same_sequence"]) <= 2e-2 * abs(dJ), (dJ, r)
    assert abs(r["fd"] - dJ) <= 4.0 * r["jump_se"], (dJ, r)
    assert 0.001 < r["changed"] / 1e6 < 0.01, r
    # the split is exact: the two parts add up to the difference of the losses
    assert abs(r["fd_jump"] + r["fd_same_sequence"] - r["fd"]) <= 1e-6 * abs(r["fd"]) + 1e-15


def test_autograd_function_matches_model():
    m = ExitEnergyModel(AL, 10000, seed=9, precision="fp64")
    t, _, _ = m.forward(1.1, 1.0)
    J = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    n = torch.tensor(1.0, dtype=torch.float64, requires_grad=True)
    h, mean = exit_histogram(J, n, m)
    L = ((h.cpu() - torch.from_numpy(t)) ** 2).sum() + 1e-8 * mean.cpu()
    L.backward()
    hh, s, nb = m.forward(1.0, 1.0)
    dJ, dn = m.backward(2.0 * (hh - t), 1e-8 / nb)
    assert abs(float(J.grad) - dJ) <= 1e-12 * abs(dJ)
    assert abs(float(n.grad) - dn) <= 1e-9 * abs(dJ)
    assert 1000.0 < float(mean) < 15000.0


# deepest z of backscattered electrons, 64 soft bins of 0-20000 A (sigma 300 A):
# the adjoint runs through the energy, the direction and the local frame
DEPTH = dict(quantity="max_depth", lo=0.0, hi=20000.0, sigma=300.0)


def test_fp64_depth_adjoint_equals_frozen_fd():
    m = ExitEnergyModel(AL, 20000, seed=13, precision="fp64", **DEPTH)
    t, _, _ = m.forward(1.1, 1.1)
    L, dJ, dn = loss_grad(m, t)
    assert L > 0
    d = 1e-5
    fdJ = (chain_loss(m, t, 1 + d) - chain_loss(m, t, 1 - d)) / (2 * d)
    fdn = (chain_loss(m, t, 1.0, 1 + d) - chain_loss(m, t, 1.0, 1 - d)) / (2 * d)
    assert abs(dJ - fdJ) <= 1e-5 * abs(fdJ), (dJ, fdJ)
    assert abs(dn - fdn) <= 1e-5 * abs(fdn), (dn, fdn)
    # unlike the exit energy, the depth scales with the density (steps ~ 1/n)
    assert abs(dn) > 0.1 * abs(dJ)


def test_fp32_depth_adjoint_against_fd_and_fp64():
    m32 = ExitEnergyModel(AL, 50000, seed=17, precision="fp32", **DEPTH)
    m64 = ExitEnergyModel(AL, 50000, seed=17, precision="fp64", **DEPTH)
    t, _, _ = m64.forward(1.1, 1.1)
    _, dJ32, dn32 = loss_grad(m32, t)
    _, dJ64, dn64 = loss_grad(m64, t)
    d = 1e-3
    fdJ = (chain_loss(m32, t, 1 + d) - chain_loss(m32, t, 1 - d)) / (2 * d)
    fdn = (chain_loss(m32, t, 1.0, 1 + d) - chain_loss(m32, t, 1.0, 1 - d)) / (2 * d)
    assert abs(dJ32 - fdJ) <= 2e-3 * abs(fdJ), (dJ32, fdJ)
    assert abs(dn32 - fdn) <= 2e-3 * abs(fdn), (dn32, fdn)
    assert abs(dJ32 - dJ64) <= 3e-2 * abs(dJ64), (dJ32, dJ64)
    assert abs(dn32 - dn64) <= 3e-2 * abs(dn64), (dn32, dn64)


def test_depth_chain_reproduces_forward():
    """At the forward's own parameters the frozen-sequence recomputation gives
    the forward's depths (it runs the same event code; the bins are sums of
    atomic additions, so their order, and the last bits, may differ)."""
    m = ExitEnergyModel(AL, 5000, seed=19, precision="fp32", **DEPTH)
    h, s, nb = m.forward(1.0, 1.0)
    hc, sc, nbc = m.chain(1.0, 1.0)
    assert nb == nbc
    assert abs(s - sc) <= 1e-12 * abs(s)
    assert np.allclose(h, hc, rtol=1e-12, atol=0.0)
