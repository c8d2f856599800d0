"""Differentiable continuous-mode transport.

ExitEnergyModel runs the continuous-slowing-down transport (mcd_adjoint_forward)
and keeps, per electron, checkpoints every 64 events.  Its backward pass
(mcd_adjoint) recomputes each 64-event segment from the Philox counters and
sweeps it in reverse, giving the pathwise derivatives of

    h_b = (1/N) sum_{bks} exp(-(q - c_b)^2 / (2 sigma^2))   (b < nbins)
    m   = mean of q over backscattered electrons

for q the exit energy (quantity="exit_E": the energy recursion
E_{k+1} = E_k - s_k S(E_k) alone) or the deepest z reached
(quantity="max_depth": energy, direction and local frame through every
Rutherford deflection up to the deepest point), with respect to the Bethe
mean ionisation energy J and the density, both as multipliers of the
reference values (J_scale, n_scale), with the random numbers and the event
sequence frozen.

exit_histogram(J_scale, n_scale, model) wraps it as a torch.autograd
Function of the two scale factors.
"""
import ctypes as C

import numpy as np

from . import _lib
from .config import with_defaults
from .engine import make_sim, _torch


SoftHist = _lib.SoftHist
AdjointBuf = _lib.AdjointBuf


class ExitEnergyModel:
    """One continuous-mode simulation whose exit-energy tallies are differentiable."""

    def __init__(self, input_par, num_el, seed=0, nbins=64, sigma=50.0, lo=None, hi=None, precision="fp32",
                 max_ckpt=64, device="cuda", quantity="exit_E"):
        torch = _torch()
        self.p = with_defaults(input_par)
        if "DS" in self.p["mode"]:
            self.p["mode"] = "cont"
        self.n = int(num_el)
        self.seed = int(seed)
        self.prec = _lib.FP64 if precision in ("fp64", _lib.FP64) else _lib.FP32
        self.device = torch.device(device)
        self.mat = _lib.material(self.p["material"])
        if quantity not in ("exit_E", "max_depth"):
            raise ValueError("quantity is 'exit_E' or 'max_depth'")
        self.depth = quantity == "max_depth"
        if self.depth and (lo is None or hi is None):
            raise ValueError("a depth histogram needs lo and hi (A)")
        lo = float(self.p["Emin"]) if lo is None else float(lo)
        hi = float(self.p["E0"]) if hi is None else float(hi)
        self.hist = SoftHist(int(nbins), _lib.ADJ_MAX_DEPTH if self.depth else _lib.ADJ_EXIT_E, lo, hi, float(sigma))
        self.nbins = int(nbins)
        self.max_ckpt = int(max_ckpt)
        self._alloc()
        self.last = None   # (J_scale, n_scale) of the stored checkpoints

    def _alloc(self):
        torch = _torch()
        dt = torch.float32 if self.prec == _lib.FP32 else torch.float64
        shape = (self.max_ckpt, 8, self.n) if self.depth else (self.max_ckpt, self.n)
        self.ckpt = torch.empty(shape, dtype=dt, device=self.device)
        self.kstar = torch.empty(self.n, dtype=torch.int32, device=self.device)
        self.E_exit = torch.empty(self.n, dtype=dt, device=self.device)
        self.queue = torch.zeros(1, dtype=torch.int64, device=self.device)   # the forward pass's work queue
        self.buf = AdjointBuf(self.ckpt.data_ptr(), self.kstar.data_ptr(), self.E_exit.data_ptr(), self.max_ckpt, 0,
                              self.queue.data_ptr())
        self.hout = torch.zeros(self.nbins + 2, dtype=torch.float64, device=self.device)
        self.status = torch.zeros(1, dtype=torch.int32, device=self.device)
        self.grad = torch.zeros(2, dtype=torch.float64, device=self.device)
        self.grad_in = torch.zeros(self.nbins + 1, dtype=torch.float64, device=self.device)

    def sim(self, J_scale, n_scale):
        return make_sim(self.p, self.n, self.seed, 0, self.prec, 0, J_scale=float(J_scale), n_scale=float(n_scale))

    def _stream(self):
        torch = _torch()
        return torch.cuda.current_stream(self.device).cuda_stream

    def launch_forward(self, J_scale=1.0, n_scale=1.0):
        """Enqueue the forward pass (no host synchronisation)."""
        self.hout.zero_()
        self.status.zero_()
        s = self.sim(J_scale, n_scale)
        code = _lib.lib().mcd_adjoint_forward(C.byref(s), C.byref(self.mat), C.byref(self.hist), C.byref(self.buf),
                                              self.hout.data_ptr(), None, self.status.data_ptr(), self._stream())
        _lib.check("mcd_adjoint_forward", code)
        self.last = (float(J_scale), float(n_scale))

    def forward(self, J_scale=1.0, n_scale=1.0):
        """Soft bins h_b (normalised by N), sum of exit energies, number of 'bks'."""
        while True:
            self.launch_forward(J_scale, n_scale)
            st = int(self.status.item())
            if not (st & _lib.FLAG_CKPT):   # an exiting electron outran the checkpoint slots
                break
            self.max_ckpt *= 2
            self._alloc()
        h = self.hout.cpu().numpy()
        return h[:self.nbins] / self.n, float(h[self.nbins]), float(h[self.nbins + 1])

    def launch_backward(self, grad_h, grad_sum):
        self.grad.zero_()
        g = np.concatenate([np.asarray(grad_h, dtype=np.float64).reshape(-1), [float(grad_sum)]])
        self.grad_in.copy_(_torch().from_numpy(g))
        s = self.sim(*self.last)
        code = _lib.lib().mcd_adjoint(C.byref(s), C.byref(self.mat), C.byref(self.hist), C.byref(self.buf),
                                      self.grad_in.data_ptr(), self.grad.data_ptr(), self._stream())
        _lib.check("mcd_adjoint", code)

    def backward(self, grad_h, grad_sum=0.0):
        """(dL/dJ_scale, dL/dn_scale) for dL/dh_b = grad_h, dL/d(sum E_exit) = grad_sum,
        at the parameters of the last forward pass."""
        if self.last is None:
            raise RuntimeError("backward before forward")
        self.launch_backward(grad_h, grad_sum)
        g = self.grad.cpu().numpy()
        return float(g[0]), float(g[1])

    def chain(self, J_scale=1.0, n_scale=1.0):
        """Soft bins and sum along the frozen event sequence of the last forward pass."""
        self.hout.zero_()
        s = self.sim(J_scale, n_scale)
        code = _lib.lib().mcd_adjoint_chain(C.byref(s), C.byref(self.mat), C.byref(self.hist), C.byref(self.buf),
                                            self.hout.data_ptr(), self._stream())
        _lib.check("mcd_adjoint_chain", code)
        h = self.hout.cpu().numpy()
        return h[:self.nbins] / self.n, float(h[self.nbins]), float(h[self.nbins + 1])


def resimulated_fd(model, target, h=1e-3, param="J"):
    """Central finite difference of L = sum_b (h_b - target_b)^2 in J_scale
    (param="J") or n_scale ("n") at 1, re-simulating at 1 -/+ h with common
    random numbers (the same Philox stream), so that an electron may take
    another event sequence -- unlike mcd_adjoint_chain, whose sequence is
    frozen.  The difference splits exactly over the electrons:

        FD = sum_e sum_b [K_b(q_e+) - K_b(q_e-)] 2 (hbar_b - t_b) / (2 h N),

    K_b the soft bin of electron e's quantity q (0 unless it backscattered),
    hbar the mean of the two runs' bins.  Electrons whose recorded event
    (kstar: the exit event, or the deepest one) is the same in both runs
    carry the smooth part the pathwise adjoint differentiates; the others
    jump, and their terms are independent across electrons, which gives the
    standard error of the jump part.  Returns a dict; the model keeps the
    checkpoints of (1, 1) afterwards."""
    torch = _torch()
    t = np.asarray(target, dtype=np.float64)
    runs = []
    for x in (1.0 - h, 1.0 + h):
        J, n = (x, 1.0) if param == "J" else (1.0, x)
        hb, _, _ = model.forward(J, n)
        runs.append((hb.copy(), model.E_exit.to(torch.float64).clone(), model.kstar.clone()))
    (hm, qm, km), (hp, qp, kp) = runs
    hist = model.hist
    centers = hist.lo + (np.arange(model.nbins) + 0.5) * (hist.hi - hist.lo) / model.nbins
    out = fd_split(qm, qp, km, kp, hm, hp, t, centers, hist.sigma, h, model.n)
    model.forward(1.0, 1.0)
    out.update(step=h, param=param)
    return out


def fd_split(qm, qp, km, kp, hm, hp, target, centers, sigma, h, n):
    """Split the central difference (L(+) - L(-)) / 2h of
    L = sum_b (h_b - t_b)^2 over the electrons.  qm/qp: per-electron
    quantity of the two runs (torch tensors, any device), km/kp: their
    recorded event (< 0 when the electron did not backscatter), hm/hp: the
    runs' soft bins (normalised by n), centers: the bin centres c_b.  With
    K_b(q) = exp(-(q - c_b)^2 / (2 sigma^2)) and hbar = (hm + hp) / 2,

        L(+) - L(-) = sum_b (hp_b - hm_b) 2 (hbar_b - t_b),
        hp_b - hm_b = (1/n) sum_e [K_b(qp_e) - K_b(qm_e)],

    so electron e carries ce_e = sum_b [K_b(qp_e) - K_b(qm_e)] 2 (hbar_b - t_b) / (2 h n),
    and the ce_e add up to the difference exactly when hm/hp are the soft
    bins of qm/qp.  Host arithmetic on the tensors' own device; no kernel of
    the transport runs here."""
    import torch
    dev = qm.device
    t = np.asarray(target, dtype=np.float64)
    fd = (float(np.sum((hp - t) ** 2)) - float(np.sum((hm - t) ** 2))) / (2.0 * h)
    cb = torch.as_tensor(np.asarray(centers, dtype=np.float64), device=dev)
    g = torch.as_tensor(2.0 * (0.5 * (hm + hp) - t), dtype=torch.float64, device=dev)
    inv2s2 = 1.0 / (2.0 * sigma * sigma)
    qm, qp = qm.to(torch.float64), qp.to(torch.float64)
    ce = torch.empty(qm.shape[0], dtype=torch.float64, device=dev)
    step = 1 << 20
    for a in range(0, qm.shape[0], step):
        b = min(qm.shape[0], a + step)
        kp_, km_ = (torch.exp(-(q[a:b, None] - cb[None, :]) ** 2 * inv2s2) @ g for q in (qp, qm))
        kp_ = torch.where(kp[a:b] >= 0, kp_, torch.zeros_like(kp_))
        km_ = torch.where(km[a:b] >= 0, km_, torch.zeros_like(km_))
        ce[a:b] = (kp_ - km_) / (2.0 * h * n)
    same = kp == km
    return {"fd": fd, "fd_same_sequence": float(ce[same].sum()), "fd_jump": float(ce[~same].sum()),
            "jump_se": float(torch.sqrt((ce[~same] ** 2).sum())), "changed": int((~same).sum())}


def _function():
    torch = _torch()

    class ExitHistogram(torch.autograd.Function):
        """(J_scale, n_scale) -> (soft bins [nbins], mean) of the model's quantity."""

        @staticmethod
        def forward(ctx, J_scale, n_scale, model):
            h, s, nb = model.forward(float(J_scale), float(n_scale))
            ctx.model = model
            ctx.nbks = max(nb, 1.0)
            ctx.devs = (J_scale.device, n_scale.device)
            dev = J_scale.device
            return (torch.as_tensor(h, dtype=torch.float64, device=dev),
                    torch.as_tensor(s / ctx.nbks, dtype=torch.float64, device=dev))

        @staticmethod
        def backward(ctx, grad_h, grad_m):
            gh = grad_h.detach().cpu().numpy() if grad_h is not None else np.zeros(ctx.model.nbins)
            gm = float(grad_m) if grad_m is not None else 0.0
            dJ, dn = ctx.model.backward(gh, gm / ctx.nbks)
            return (torch.as_tensor(dJ, dtype=torch.float64, device=ctx.devs[0]),
                    torch.as_tensor(dn, dtype=torch.float64, device=ctx.devs[1]), None)

    return ExitHistogram


_FN = None


def exit_histogram(J_scale, n_scale, model):
    """Differentiable (soft bins, mean) of the model's quantity (exit energy
    or deepest z of the backscattered electrons) for torch scalars J_scale,
    n_scale."""
    global _FN
    if _FN is None:
        _FN = _function()
    return _FN.apply(J_scale, n_scale, model)
