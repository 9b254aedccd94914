"""Gradients of liquid water and surface rain through the condensation and
grid-advection sub-steps.

Two differentiated models share the adjoint kernels (csrc/k_adjoint.cu):

``StepModel(st, n_adv)`` runs the product's own FP64 time step
(integration.py:1298-1612, collisions off) for ``n_adv`` advection steps and
records each SIP's cell at every particle sub-step.  Its forward model replays
that run with the recorded cells: per half step the advective (+ relaxation)
increments of Theta and r_v (integration.py:1483-1508, 1536-1561), per
sub-step the condensation map of every SIP (the time step's own damped Newton
of ``no_iter_impl_mass`` evaluations, integration.py:786-836, or the implicit
step solved to convergence) and the cell update (integration.py:402-438).  SIP
motion, ground removal and re-indexing enter only through the piecewise
constant cell index and are held fixed; so are multiplicities.  With the
recorded cells the forward model reproduces the product's run.

``CondensationModel(st)`` is the condensation-only model: cells fixed at their
initial values and no advection.

``objective(model, m_s, kappa, flux_scale, weights, ...)`` returns J = sum_k
weights_k m_w,k after the run as a torch scalar whose backward pass is the
hand-written adjoint (reverse sweep per sub-step, the increments' Jacobian
per half step, checkpoints every ``checkpoint_every`` advection steps, each
segment recomputed from its stored start).  Gradients flow to ``m_s`` (per SIP
solute mass, fg), ``kappa`` (the hygroscopicity that scales the ammonium-
sulfate water activity, a_w = 1 + (kappa / 0.6)(a_w_AS - 1); kappa = 0.6 is
the reference's a_w) and ``flux_scale`` (a common factor of the mass flux,
i.e. of j_max at init.py:1146-1148; dJ/dj_max = dJ/dflux_scale / j_max).
``StepModel.lwp_weights()`` and ``rain_weights()`` give the domain-mean liquid
water path at the end and the mean surface rain flux over the run (the SIPs
removed at the ground, integration.py:606-630, whose masses froze at removal).
"""

import numpy as np
import torch

from . import _lib
from .device import DeviceState, _ptr, _stream, to_device

F64 = torch.float64


class _Base:
    def _common(self, st, dev):
        self.lib = _lib.load()
        nx, nz = (int(v) for v in st["grid_no_cells"])
        self.nx, self.nz, self.C = nx, nz, nx * nz
        self.m_s0 = to_device(st["m_s"], device=dev)
        self.xi = to_device(st["xi"], device=dev)
        self.n = int(self.xi.numel())
        gsf = np.asarray(st["grid_scalar_fields"])
        self.rho_d = to_device(gsf[3].ravel(), device=dev)
        self.mdi = to_device(gsf[8].ravel(), device=dev)
        self.rdi = to_device(gsf[9].ravel(), device=dev)
        self.dml = torch.zeros(self.C, dtype=F64, device=dev)
        self.dt_sub = float(st["dt_sub"])
        self.p_ref = float(st["p_ref"])
        self.V = float(st["grid_volume_cell"])
        self.dx, self.dz = (float(v) for v in np.asarray(st["grid_steps"]))
        self.no_iter = int(st["no_iter_impl_mass"])

    def _sub_steps(self, m_w, m_s, Th, rv, kappa, cell, stride, n_sub, inc, no_iter,
                   tape_m=None, tape_c=None):
        _lib.check(self.lib.lacmo_adj_forward(
            self.n, self.C, _ptr(m_w), _ptr(m_s), _ptr(self.xi), _ptr(cell), int(stride),
            _ptr(Th), _ptr(rv), _ptr(self.rho_d), _ptr(self.mdi),
            _ptr(inc[0]) if inc is not None else None, _ptr(inc[1]) if inc is not None else None,
            _ptr(self.dml), self.dt_sub, float(kappa), self.p_ref, self.V, int(n_sub),
            int(no_iter), _ptr(tape_m), _ptr(tape_c), _stream()), "adj_forward")

    def _sub_steps_bwd(self, m_s, kappa, cell, stride, n_sub, inc, no_iter, tape_m, tape_c, lam,
                       grad_ms, grad_k, lam_inc):
        lam_m, lam_Th, lam_rv, lam_dml = lam
        _lib.check(self.lib.lacmo_adj_backward(
            self.n, self.C, _ptr(m_s), _ptr(self.xi), _ptr(cell), int(stride), _ptr(self.rho_d),
            _ptr(self.mdi), _ptr(inc[0]) if inc is not None else None,
            _ptr(inc[1]) if inc is not None else None, _ptr(self.dml), self.dt_sub,
            float(kappa), self.p_ref, self.V, int(n_sub), int(no_iter), _ptr(tape_m),
            _ptr(tape_c), _ptr(lam_m), _ptr(lam_Th), _ptr(lam_rv), _ptr(lam_dml),
            _ptr(grad_ms), _ptr(grad_k), _ptr(lam_inc), _stream()), "adj_backward")


class CondensationModel(_Base):
    """Condensation only: cells fixed at their initial values, no advection;
    each sub-step's implicit step solved to convergence (``no_iter`` 0) unless
    ``no_iter`` is given."""

    def __init__(self, st, device="cuda", no_iter=0):
        self._common(st, device)
        cells = np.asarray(st["cells"])
        act = np.asarray(st["active_ids"], dtype=bool)
        cell = np.where(act, cells[0] * self.nz + cells[1], -1).astype(np.int32)
        self.cell = torch.from_numpy(cell).to(device)
        self.m_w0 = to_device(st["m_w"], device=device)
        gsf = np.asarray(st["grid_scalar_fields"])
        self.Th0 = to_device(gsf[2].ravel(), device=device)
        self.rv0 = to_device(gsf[4].ravel(), device=device)
        self.no_iter = int(no_iter)

    def lwp_weights(self):
        """Weights of the domain-mean liquid water path (kg m^-2 per fg of
        m_w): xi * 1e-18 over the domain's horizontal extent (unit depth)."""
        w = self.xi * 1.0E-18 / (self.nx * self.dx)
        return torch.where(self.cell >= 0, w, torch.zeros_like(w))

    def _forward(self, m_w, m_s, Th, rv, kappa, n_sub, tape_m=None, tape_c=None):
        self._sub_steps(m_w, m_s, Th, rv, kappa, self.cell, 0, n_sub, None, self.no_iter,
                        tape_m, tape_c)

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
        dev = m_s.device
        lam = ((weights * gJ).contiguous().clone(), torch.zeros(C, dtype=F64, device=dev),
               torch.zeros(C, dtype=F64, device=dev), torch.zeros(C, dtype=F64, device=dev))
        grad_ms = torch.zeros(n, dtype=F64, device=dev)
        grad_k = torch.zeros(1, dtype=F64, device=dev)
        for m_w0, Th0, rv0, seg in reversed(ctx.checkpoints):
            tape_m = torch.empty((seg + 1) * n, dtype=F64, device=dev)
            tape_c = torch.empty(seg * 2 * C, dtype=F64, device=dev)
            m_w, Th, rv = m_w0.clone(), Th0.clone(), rv0.clone()
            model._forward(m_w, m_s, Th, rv, k, seg, tape_m, tape_c)
            model._sub_steps_bwd(m_s, k, model.cell, 0, seg, None, model.no_iter, tape_m, tape_c,
                                 lam, grad_ms, grad_k, None)
        return grad_ms, grad_k[0], None, None, None, None


def liquid_water(model, m_s, kappa, weights=None, n_sub=10, checkpoint_every=600):
    """J = sum(weights * m_w) after n_sub sub-steps of a CondensationModel,
    differentiable in m_s (tensor [n], fg) and kappa (0-d tensor); weights
    default to the domain-mean liquid water path."""
    if weights is None:
        weights = model.lwp_weights()
    if not isinstance(kappa, torch.Tensor):
        kappa = torch.tensor(float(kappa), dtype=F64, device=m_s.device)
    return _LiquidWater.apply(m_s, kappa, model, weights, int(n_sub), int(checkpoint_every))


class StepModel(_Base):
    """The product's time step replayed with recorded cells (module
    docstring).  ``st``: a state dict of the drop-in layer; ``n_adv``
    advection steps are run once by the product (FP64, collisions off) to
    record the cells; ``self.product`` keeps that run's final DeviceState."""

    def __init__(self, st, n_adv, device="cuda"):
        self._common(st, device)
        self.n_adv = int(n_adv)
        self.dt = float(st["dt"])
        self.S = int(st["scale_dt_cond"])
        self.K = 2 * self.S * self.n_adv
        gsf = np.asarray(st["grid_scalar_fields"])
        self.m_w0 = to_device(st["m_w"], device=device)
        self.Th0 = to_device(gsf[2].ravel(), device=device)
        self.rv0 = to_device(gsf[4].ravel(), device=device)
        self.flux = to_device(st["grid_mass_flux_air_dry"], device=device).contiguous()
        self.relax = bool(st["act_relaxation"]) and st.get("init_profile_r_v") is not None
        if self.relax:
            self.prof_th = to_device(st["init_profile_Theta"], device=device)
            self.prof_rv = to_device(st["init_profile_r_v"], device=device)
            self.t_relax = to_device(st["relaxation_time_profile"], device=device)
        st_run = dict(st)
        st_run["act_collisions"] = False
        ds = DeviceState(st_run, device=device)
        self.cells = torch.empty((self.K, self.n), dtype=torch.int32, device=device)
        self.cell_start = ds.cell.clone()
        for a in range(self.n_adv):
            base = 2 * self.S * a
            ds.adv_step_tracked(lambda k: self.cells[base + k].copy_(ds.cell))
        self.cell_end = ds.cell.clone()
        self.product = ds

    # -- objectives ---------------------------------------------------------------
    def lwp_weights(self):
        """Domain-mean liquid water path at the end (kg m^-2 per fg of m_w)."""
        w = self.xi * 1.0E-18 / (self.nx * self.dx)
        return torch.where(self.cell_end >= 0, w, torch.zeros_like(w))

    def rain_weights(self):
        """Mean surface rain flux over the run (kg m^-2 s^-1 per fg of m_w):
        the water of the SIPs in the domain at the start and removed at the
        ground by the end (water_removed, integration.py:617-628), per
        domain width and run time."""
        w = self.xi * 1.0E-18 / (self.nx * self.dx * self.n_adv * self.dt)
        removed = (self.cell_start >= 0) & (self.cell_end < 0)
        return torch.where(removed, w, torch.zeros_like(w))

    # -- forward ------------------------------------------------------------------
    def _inc_args(self, Th, rv, flux):
        return (_ptr(Th), _ptr(rv), _ptr(self.rdi), _ptr(flux), self.nx, self.nz, self.dx,
                self.dz, self.dt_sub, _ptr(self.prof_th) if self.relax else None,
                _ptr(self.prof_rv) if self.relax else None,
                _ptr(self.t_relax) if self.relax else None)

    def _increments(self, Th, rv, flux, second, inc):
        _lib.check(self.lib.lacmo_adj_increments(*self._inc_args(Th, rv, flux), int(second),
                                                 _ptr(inc[0]), _ptr(inc[1]), _stream()),
                   "adj_increments")

    def _half(self, a, h, m_w, m_s, Th, rv, kappa, inc, no_iter, tape_m=None, tape_c=None):
        k0 = (2 * a + h) * self.S
        self._sub_steps(m_w, m_s, Th, rv, kappa, self.cells[k0], self.n, self.S, inc, no_iter,
                        tape_m, tape_c)

    def _adv(self, a, m_w, m_s, Th, rv, kappa, flux, no_iter):
        inc = torch.empty((2, self.C), dtype=F64, device=m_w.device)
        self._increments(Th, rv, flux, 0, inc)
        self._half(a, 0, m_w, m_s, Th, rv, kappa, inc, no_iter)
        self._increments(Th, rv, flux, 1, inc)
        self._half(a, 1, m_w, m_s, Th, rv, kappa, inc, no_iter)

    def scaled_flux(self, flux_scale):
        s = float(flux_scale)
        return self.flux if s == 1.0 else self.flux * s

    def run(self, m_s=None, kappa=0.6, flux_scale=1.0, no_iter=None, starts=None, a0=0,
            a1=None, state=None):
        """Forward model over advection steps a0 .. a1 - 1 (default: all) from
        ``state`` = (m_w, Theta, r_v) (default: the initial state); returns the
        final (m_w, Theta, r_v).  ``starts`` (a list) collects the state at the
        start of every step."""
        m_s = (self.m_s0 if m_s is None else m_s).detach().contiguous()
        no_iter = self.no_iter if no_iter is None else int(no_iter)
        flux = self.scaled_flux(flux_scale)
        m_w, Th, rv = (t.clone() for t in (state or (self.m_w0, self.Th0, self.rv0)))
        for a in range(a0, self.n_adv if a1 is None else a1):
            if starts is not None:
                starts.append((m_w.clone(), Th.clone(), rv.clone()))
            self._adv(a, m_w, m_s, Th, rv, float(kappa), flux, no_iter)
        return m_w, Th, rv

    # -- reverse ------------------------------------------------------------------
    def _adv_bwd(self, a, start, m_s, kappa, flux, flux_scale, no_iter, lam, grad_ms, grad_k,
                 grad_s):
        """Reverse of advection step a from its start state; lam holds the
        adjoints after the step on entry and before it on return."""
        n, C, S = self.n, self.C, self.S
        dev = m_s.device
        m_w, Th, rv = (t.clone() for t in start)
        Th_a, rv_a = Th.clone(), rv.clone()
        inc1 = torch.empty((2, C), dtype=F64, device=dev)
        self._increments(Th, rv, flux, 0, inc1)
        tapes = [(torch.empty((S + 1) * n, dtype=F64, device=dev),
                  torch.empty(S * 2 * C, dtype=F64, device=dev)) for _ in range(2)]
        self._half(a, 0, m_w, m_s, Th, rv, kappa, inc1, no_iter, *tapes[0])
        Th_m, rv_m = Th.clone(), rv.clone()
        inc2 = inc1.clone()
        self._increments(Th, rv, flux, 1, inc2)
        self._half(a, 1, m_w, m_s, Th, rv, kappa, inc2, no_iter, *tapes[1])
        lam_inc = torch.zeros((2, C), dtype=F64, device=dev)
        k1 = (2 * a + 1) * S
        self._sub_steps_bwd(m_s, kappa, self.cells[k1], n, S, inc2, no_iter, *tapes[1], lam,
                            grad_ms, grad_k, lam_inc)
        # inc2 = 2 inc(mid) - inc1
        self._vjp(Th_m, rv_m, flux, 2.0, flux_scale, lam_inc, lam, grad_s)
        lam_inc.neg_()
        k0 = 2 * a * S
        self._sub_steps_bwd(m_s, kappa, self.cells[k0], n, S, inc1, no_iter, *tapes[0], lam,
                            grad_ms, grad_k, lam_inc)
        self._vjp(Th_a, rv_a, flux, 1.0, flux_scale, lam_inc, lam, grad_s)

    def _vjp(self, Th, rv, flux, factor, flux_scale, lam_inc, lam, grad_s):
        _lib.check(self.lib.lacmo_adj_increments_vjp(
            *self._inc_args(Th, rv, flux), float(factor), float(flux_scale), _ptr(lam_inc),
            _ptr(lam[1]), _ptr(lam[2]), _ptr(grad_s), _stream()), "adj_increments_vjp")


class _StepObjective(torch.autograd.Function):
    @staticmethod
    def forward(ctx, m_s, kappa, flux_scale, model, weights, no_iter, every):
        m_s = m_s.detach().contiguous()
        k, s = float(kappa), float(flux_scale)
        ni = model.no_iter if no_iter is None else int(no_iter)
        flux = model.scaled_flux(s)
        m_w, Th, rv = model.m_w0.clone(), model.Th0.clone(), model.rv0.clone()
        checkpoints = []
        for a in range(model.n_adv):
            if a % every == 0:
                checkpoints.append((a, (m_w.clone(), Th.clone(), rv.clone())))
            model._adv(a, m_w, m_s, Th, rv, k, flux, ni)
        ctx.model, ctx.checkpoints, ctx.k, ctx.s, ctx.ni = model, checkpoints, k, s, ni
        ctx.every = every
        ctx.save_for_backward(m_s, weights)
        return (weights * m_w).sum()

    @staticmethod
    def backward(ctx, gJ):
        m_s, weights = ctx.saved_tensors
        model, k, s, ni = ctx.model, ctx.k, ctx.s, ctx.ni
        dev = m_s.device
        C = model.C
        flux = model.scaled_flux(s)
        lam = ((weights * gJ).contiguous().clone(), torch.zeros(C, dtype=F64, device=dev),
               torch.zeros(C, dtype=F64, device=dev), torch.zeros(C, dtype=F64, device=dev))
        grad_ms = torch.zeros(model.n, dtype=F64, device=dev)
        grad_k = torch.zeros(1, dtype=F64, device=dev)
        grad_s = torch.zeros(1, dtype=F64, device=dev)
        for a0, state in reversed(ctx.checkpoints):
            a1 = min(a0 + ctx.every, model.n_adv)
            starts = []
            model.run(m_s, k, s, ni, starts=starts, a0=a0, a1=a1, state=state)
            for a in range(a1 - 1, a0 - 1, -1):
                model._adv_bwd(a, starts[a - a0], m_s, k, flux, s, ni, lam, grad_ms, grad_k,
                               grad_s)
        return grad_ms, grad_k[0], grad_s[0], None, None, None, None


def objective(model, m_s, kappa, flux_scale=1.0, weights=None, no_iter=None,
              checkpoint_every=10):
    """J = sum(weights * m_w) after the StepModel's run, differentiable in
    m_s (tensor [n], fg), kappa and flux_scale (0-d tensors or floats);
    weights default to the liquid water path at the end; no_iter None: the
    state's own Newton count, 0: the implicit step solved to convergence."""
    dev = m_s.device
    if weights is None:
        weights = model.lwp_weights()
    if not isinstance(kappa, torch.Tensor):
        kappa = torch.tensor(float(kappa), dtype=F64, device=dev)
    if not isinstance(flux_scale, torch.Tensor):
        flux_scale = torch.tensor(float(flux_scale), dtype=F64, device=dev)
    return _StepObjective.apply(m_s, kappa, flux_scale, model, weights, no_iter,
                                int(checkpoint_every))
