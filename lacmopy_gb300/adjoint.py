"""Gradients of liquid water through the condensation sub-steps.

``CondensationModel`` holds a 2-D state on the GPU in the form the adjoint
kernels (csrc/k_adjoint.cu) differentiate: SIP masses with fixed cells and
multiplicities, the cells' Theta and r_v with their dry density, and the
sub-step length.  Collisions and SIP motion are recorded events held fixed;
every sub-step solves the implicit Euler condensation step of each SIP
(integration.py:728-836) to convergence and feeds the condensed mass back into
Theta and r_v (integration.py:402-438).

``liquid_water(model, m_s, kappa, weights, n_sub, checkpoint_every)`` returns
J = sum_k weights_k m_w,k after ``n_sub`` sub-steps as a torch scalar whose
backward pass is the hand-written adjoint: the implicit-function theorem
through each SIP's root and the reverse sweep over sub-steps, recomputing
each segment of ``checkpoint_every`` sub-steps from its stored start state.
Gradients flow to ``m_s`` (per SIP solute mass, fg) and ``kappa`` (the
hygroscopicity that scales the ammonium-sulfate water activity, a_w = 1 +
(kappa / 0.6)(a_w_AS - 1); kappa = 0.6 is the reference's a_w).
"""

import numpy as np
import torch

from . import _lib
from .device import _ptr, _stream, to_device

F64 = torch.float64


class CondensationModel:
    def __init__(self, st, device="cuda"):
        self.lib = _lib.load()
        nx, nz = (int(v) for v in st["grid_no_cells"])
        self.nx, self.nz, self.C = nx, nz, nx * nz
        cells = np.asarray(st["cells"])
        act = np.asarray(st["active_ids"], dtype=bool)
        cell = np.where(act, cells[0] * nz + cells[1], -1).astype(np.int32)
        self.n = int(cell.size)
        dev = device
        self.m_w0 = to_device(st["m_w"], device=dev)
        self.m_s0 = to_device(st["m_s"], device=dev)
        self.xi = to_device(st["xi"], device=dev)
        self.cell = torch.from_numpy(cell).to(dev)
        gsf = np.asarray(st["grid_scalar_fields"])
        self.Th0 = to_device(gsf[2].ravel(), device=dev)
        self.rv0 = to_device(gsf[4].ravel(), device=dev)
        self.rho_d = to_device(gsf[3].ravel(), device=dev)
        self.mdi = to_device(gsf[8].ravel(), device=dev)
        self.dml = torch.zeros(self.C, dtype=F64, device=dev)
        self.dt_sub = float(st["dt_sub"])
        self.p_ref = float(st["p_ref"])
        self.V = float(st["grid_volume_cell"])
        self.dx = float(np.asarray(st["grid_steps"])[0])

    def lwp_weights(self):
        """Weights of the domain-mean liquid water path (kg m^-2 per fg of
        m_w): xi * 1e-18 over the domain's horizontal extent (unit depth)."""
        w = self.xi * 1.0E-18 / (self.nx * self.dx)
        return torch.where(self.cell >= 0, w, torch.zeros_like(w))

    def _forward(self, m_w, m_s, Th, rv, kappa, n_sub, tape_m=None, tape_c=None):
        _lib.check(self.lib.lacmo_adj_forward(
            self.n, self.C, _ptr(m_w), _ptr(m_s), _ptr(self.xi), _ptr(self.cell), _ptr(Th),
            _ptr(rv), _ptr(self.rho_d), _ptr(self.mdi), None, None, _ptr(self.dml),
            self.dt_sub, float(kappa), self.p_ref, self.V, int(n_sub), _ptr(tape_m),
            _ptr(tape_c), _stream()), "adj_forward")

    def run(self, m_s, kappa, n_sub):
        """Plain forward: the final (m_w, Theta, r_v)."""
        m_w, Th, rv = self.m_w0.clone(), self.Th0.clone(), self.rv0.clone()
        self._forward(m_w, m_s.detach().contiguous(), Th, rv, kappa, n_sub)
        return m_w, Th, rv


class _LiquidWater(torch.autograd.Function):
    @staticmethod
    def forward(ctx, m_s, kappa, model, weights, n_sub, every):
        m_s = m_s.detach().contiguous()
        k = float(kappa)
        m_w, Th, rv = model.m_w0.clone(), model.Th0.clone(), model.rv0.clone()
        checkpoints = []
        done = 0
        while done < n_sub:
            seg = min(every, n_sub - done)
            checkpoints.append((m_w.clone(), Th.clone(), rv.clone(), seg))
            model._forward(m_w, m_s, Th, rv, k, seg)
            done += seg
        ctx.model, ctx.checkpoints, ctx.kappa = model, checkpoints, k
        ctx.save_for_backward(m_s, weights)
        return (weights * m_w).sum()

    @staticmethod
    def backward(ctx, gJ):
        m_s, weights = ctx.saved_tensors
        model, k = ctx.model, ctx.kappa
        n, C = model.n, model.C
        lam_m = (weights * gJ).contiguous().clone()
        lam_Th = torch.zeros(C, dtype=F64, device=m_s.device)
        lam_rv = torch.zeros(C, dtype=F64, device=m_s.device)
        lam_dml = torch.zeros(C, dtype=F64, device=m_s.device)
        grad_ms = torch.zeros(n, dtype=F64, device=m_s.device)
        grad_k = torch.zeros(1, dtype=F64, device=m_s.device)
        for m_w0, Th0, rv0, seg in reversed(ctx.checkpoints):
            tape_m = torch.empty((seg + 1) * n, dtype=F64, device=m_s.device)
            tape_c = torch.empty(seg * 2 * C, dtype=F64, device=m_s.device)
            m_w, Th, rv = m_w0.clone(), Th0.clone(), rv0.clone()
            model._forward(m_w, m_s, Th, rv, k, seg, tape_m, tape_c)
            _lib.check(model.lib.lacmo_adj_backward(
                n, C, _ptr(m_s), _ptr(model.xi), _ptr(model.cell), _ptr(model.rho_d),
                _ptr(model.mdi), None, None, _ptr(model.dml), model.dt_sub, k, model.p_ref,
                model.V, seg, _ptr(tape_m), _ptr(tape_c), _ptr(lam_m), _ptr(lam_Th),
                _ptr(lam_rv), _ptr(lam_dml), _ptr(grad_ms), _ptr(grad_k), _stream()),
                "adj_backward")
        return grad_ms, grad_k[0], None, None, None, None


def liquid_water(model, m_s, kappa, weights=None, n_sub=10, checkpoint_every=600):
    """J = sum(weights * m_w) after n_sub sub-steps, differentiable in m_s
    (tensor [n], fg) and kappa (0-d tensor); weights default to the
    domain-mean liquid water path."""
    if weights is None:
        weights = model.lwp_weights()
    if not isinstance(kappa, torch.Tensor):
        kappa = torch.tensor(float(kappa), dtype=F64, device=m_s.device)
    return _LiquidWater.apply(m_s, kappa, model, weights, int(n_sub), int(checkpoint_every))
