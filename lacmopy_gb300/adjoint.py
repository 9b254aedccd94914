"""Gradients of liquid water and surface rain through the condensation and
grid-advection sub-steps.

Two differentiated models share the adjoint kernels (csrc/k_adjoint.cu):

``StepModel(st, n_adv)`` runs the product's own FP64 time step
(integration.py:1298-1612) for ``n_adv`` advection steps and records each
SIP's cell at every particle sub-step and every collection of every collision
step.  Its forward model replays that run: per half step the advective (+
relaxation) increments of Theta and r_v (integration.py:1483-1508,
1536-1561), the recorded collections (collision/all_or_nothing.py:577-633:
the collected masses added, p_crit times them for a multiple collection, or
an equal-multiplicity pair split), per sub-step the condensation map of every
SIP (the time step's own damped Newton of ``no_iter_impl_mass`` evaluations,
integration.py:786-836, or the implicit step solved to convergence) and the
cell update (integration.py:402-438).  SIP motion, ground removal and
re-indexing enter only through the piecewise constant cell index, and the
collision decisions, p_crit and multiplicities are recorded: all are held
fixed.  The forward model reproduces the product's run.

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
                   tape_m=None, tape_c=None, xi=None):
        xi = self.xi if xi is None else xi
        _lib.check(self.lib.lacmo_adj_forward(
            self.n, self.C, _ptr(m_w), _ptr(m_s), _ptr(xi), _ptr(cell), int(stride),
            _ptr(Th), _ptr(rv), _ptr(self.rho_d), _ptr(self.mdi),
            _ptr(inc[0]) if inc is not None else None, _ptr(inc[1]) if inc is not None else None,
            _ptr(self.dml), self.dt_sub, float(kappa), self.p_ref, self.V, int(n_sub),
            int(no_iter), _ptr(tape_m), _ptr(tape_c), _stream()), "adj_forward")

    def _sub_steps_bwd(self, m_s, kappa, cell, stride, n_sub, inc, no_iter, tape_m, tape_c, lam,
                       grad_ms, grad_k, lam_inc, xi=None):
        xi = self.xi if xi is None else xi
        lam_m, lam_Th, lam_rv, lam_dml = lam
        _lib.check(self.lib.lacmo_adj_backward(
            self.n, self.C, _ptr(m_s), _ptr(xi), _ptr(cell), int(stride), _ptr(self.rho_d),
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
    """The product's time step replayed with recorded cells and collisions
    (module docstring).  ``st``: a state dict of the drop-in layer; ``n_adv``
    advection steps are run once by the product (FP64; with collisions when
    ``collisions`` is true, default the state's own setting) to record every
    SIP's cell before each particle sub-step and every collection of each
    collision step; ``self.product`` keeps that run's final DeviceState."""

    def __init__(self, st, n_adv, device="cuda", collisions=None, log_capacity=1 << 22):
        self._common(st, device)
        self.n_adv = int(n_adv)
        self.dt = float(st["dt"])
        self.S = int(st["scale_dt_cond"])
        self.K = 2 * self.S * self.n_adv
        gsf = np.asarray(st["grid_scalar_fields"])
        self.m_w0 = to_device(st["m_w"], device=device)
        self.xi0 = self.xi
        self.Th0 = to_device(gsf[2].ravel(), device=device)
        self.rv0 = to_device(gsf[4].ravel(), device=device)
        self.flux = to_device(st["grid_mass_flux_air_dry"], device=device).contiguous()
        self.relax = bool(st["act_relaxation"]) and st.get("init_profile_r_v") is not None
        if self.relax:
            self.prof_th = to_device(st["init_profile_Theta"], device=device)
            self.prof_rv = to_device(st["init_profile_r_v"], device=device)
            self.t_relax = to_device(st["relaxation_time_profile"], device=device)
        self.collisions = bool(st["act_collisions"]) if collisions is None else bool(collisions)
        st_run = dict(st)
        st_run["act_collisions"] = self.collisions
        ds = DeviceState(st_run, device=device)
        self.cells = torch.empty((self.K, self.n), dtype=torch.int32, device=device)
        self.events = {}   # sub-step k -> [(records [r][32] uint8, offsets [G + 1], G), ...]
        self.n_events = 0
        self.cell_start = ds.cell.clone()
        log = cnt = None
        if self.collisions:
            log = torch.empty(int(log_capacity) * 32, dtype=torch.uint8, device=device)
            cnt = torch.zeros(1, dtype=torch.int64, device=device)
            _lib.check(self.lib.lacmo_collision_event_log(_ptr(log), int(log_capacity),
                                                          _ptr(cnt)), "collision_event_log")
        try:
            for a in range(self.n_adv):
                base = 2 * self.S * a

                def collide(k, step, base=base):
                    cnt.zero_()
                    step()
                    self._keep_events(base + k, log, int(cnt.item()), int(log_capacity),
                                      ds.cell)

                ds.adv_step_tracked(lambda k, base=base: self.cells[base + k].copy_(ds.cell),
                                    collide if self.collisions else None)
        finally:
            if self.collisions:
                self.lib.lacmo_collision_event_log(None, 0, None)
        self.cell_end = ds.cell.clone()
        self.xi_end = ds.xi.clone()
        self.product = ds

    def _keep_events(self, k, log, count, capacity, cell):
        """The records of one collision step before sub-step k, grouped by the
        cell of their SIPs (a cell's records keep their order)."""
        if count > capacity:
            raise _lib.LacmoError(f"collision event log: {count} records, capacity {capacity}")
        if count == 0:
            return
        rec = log[:count * 32].view(count, 32)
        imin = rec.view(torch.int32)[:, 0].long()
        key = cell[imin].long()
        order = torch.sort(key, stable=True).indices
        rec = rec[order].contiguous()
        _, cnts = torch.unique_consecutive(key[order], return_counts=True)
        off = torch.zeros(cnts.numel() + 1, dtype=torch.int64, device=rec.device)
        off[1:] = torch.cumsum(cnts, 0)
        self.events.setdefault(k, []).append((rec, off, int(cnts.numel())))
        self.n_events += count

    # -- objectives ---------------------------------------------------------------
    def lwp_weights(self):
        """Domain-mean liquid water path at the end (kg m^-2 per fg of m_w;
        the multiplicities at the end)."""
        w = self.xi_end * 1.0E-18 / (self.nx * self.dx)
        return torch.where(self.cell_end >= 0, w, torch.zeros_like(w))

    def rain_weights(self):
        """Mean surface rain flux over the run (kg m^-2 s^-1 per fg of m_w):
        the water of the SIPs in the domain at the start and removed at the
        ground by the end (water_removed, integration.py:617-628), per
        domain width and run time."""
        w = self.xi_end * 1.0E-18 / (self.nx * self.dx * self.n_adv * self.dt)
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

    def _chunks(self, a, h):
        """The half step's sub-steps cut at its collision steps: (k0, k1) runs
        of global sub-steps, each after the collisions recorded before k0."""
        lo = (2 * a + h) * self.S
        hi = lo + self.S
        cuts = sorted(k for k in self.events if lo < k < hi)
        edges = [lo] + cuts + [hi]
        return list(zip(edges[:-1], edges[1:]))

    def _collide(self, k, state):
        m_w, m_s, xi = state[0], state[1], state[2]
        for rec, off, G in self.events.get(k, ()):
            _lib.check(self.lib.lacmo_adj_collisions_forward(
                _ptr(rec), _ptr(off), G, _ptr(m_w), _ptr(m_s), _ptr(xi), _stream()),
                "adj_collisions_forward")

    def _half(self, a, h, state, kappa, inc, no_iter, tapes=None):
        """Advance ``state`` = [m_w, m_s, xi, Theta, r_v] over half step h of
        advection step a; with ``tapes`` (a list) each run of sub-steps
        appends (k0, k1, m_s, xi, tape_m, tape_c) for the reverse sweep."""
        m_w, m_s, xi, Th, rv = state
        for k0, k1 in self._chunks(a, h):
            self._collide(k0, state)
            nk = k1 - k0
            tm = tc = None
            if tapes is not None:
                tm = torch.empty((nk + 1) * self.n, dtype=F64, device=m_w.device)
                tc = torch.empty(nk * 2 * self.C, dtype=F64, device=m_w.device)
                tapes.append((k0, k1, m_s.clone(), xi.clone(), tm, tc))
            self._sub_steps(m_w, m_s, Th, rv, kappa, self.cells[k0], self.n, nk, inc, no_iter,
                            tm, tc, xi=xi)

    def _adv(self, a, state, kappa, flux, no_iter):
        Th, rv = state[3], state[4]
        inc = torch.empty((2, self.C), dtype=F64, device=Th.device)
        self._increments(Th, rv, flux, 0, inc)
        self._half(a, 0, state, kappa, inc, no_iter)
        self._increments(Th, rv, flux, 1, inc)
        self._half(a, 1, state, kappa, inc, no_iter)

    def scaled_flux(self, flux_scale):
        s = float(flux_scale)
        return self.flux if s == 1.0 else self.flux * s

    def initial_state(self, m_s=None):
        m_s = (self.m_s0 if m_s is None else m_s).detach()
        return [self.m_w0.clone(), m_s.clone().contiguous(), self.xi0.clone(), self.Th0.clone(),
                self.rv0.clone()]

    def run(self, m_s=None, kappa=0.6, flux_scale=1.0, no_iter=None, starts=None, a0=0,
            a1=None, state=None, full=False):
        """Forward model over advection steps a0 .. a1 - 1 (default: all) from
        ``state`` = [m_w, m_s, xi, Theta, r_v] (default: the initial state with
        solute masses m_s); returns the final (m_w, Theta, r_v), or the whole
        final state when ``full``.  ``starts`` (a list) collects the state at
        the start of every step."""
        no_iter = self.no_iter if no_iter is None else int(no_iter)
        flux = self.scaled_flux(flux_scale)
        st = [t.clone() for t in state] if state is not None else self.initial_state(m_s)
        for a in range(a0, self.n_adv if a1 is None else a1):
            if starts is not None:
                starts.append([t.clone() for t in st])
            self._adv(a, st, float(kappa), flux, no_iter)
        return st if full else (st[0], st[3], st[4])

    # -- reverse ------------------------------------------------------------------
    def _adv_bwd(self, a, start, kappa, flux, flux_scale, no_iter, lam, grad_ms, grad_k,
                 grad_s):
        """Reverse of advection step a from its start state; lam and grad_ms
        (the adjoint of the current solute masses) hold the adjoints after the
        step on entry and before it on return."""
        st = [t.clone() for t in start]
        Th, rv = st[3], st[4]
        Th_a, rv_a = Th.clone(), rv.clone()
        C = self.C
        inc1 = torch.empty((2, C), dtype=F64, device=Th.device)
        self._increments(Th, rv, flux, 0, inc1)
        tapes0, tapes1 = [], []
        self._half(a, 0, st, kappa, inc1, no_iter, tapes0)
        Th_m, rv_m = Th.clone(), rv.clone()
        inc2 = inc1.clone()
        self._increments(Th, rv, flux, 1, inc2)
        self._half(a, 1, st, kappa, inc2, no_iter, tapes1)
        lam_inc = torch.zeros((2, C), dtype=F64, device=Th.device)
        self._half_bwd(tapes1, kappa, inc2, no_iter, lam, grad_ms, grad_k, lam_inc)
        # inc2 = 2 inc(mid) - inc1
        self._vjp(Th_m, rv_m, flux, 2.0, flux_scale, lam_inc, lam, grad_s)
        lam_inc.neg_()
        self._half_bwd(tapes0, kappa, inc1, no_iter, lam, grad_ms, grad_k, lam_inc)
        self._vjp(Th_a, rv_a, flux, 1.0, flux_scale, lam_inc, lam, grad_s)

    def _half_bwd(self, tapes, kappa, inc, no_iter, lam, grad_ms, grad_k, lam_inc):
        for k0, k1, m_s, xi, tm, tc in reversed(tapes):
            self._sub_steps_bwd(m_s, kappa, self.cells[k0], self.n, k1 - k0, inc, no_iter, tm,
                                tc, lam, grad_ms, grad_k, lam_inc, xi=xi)
            for rec, off, G in reversed(self.events.get(k0, ())):
                _lib.check(self.lib.lacmo_adj_collisions_backward(
                    _ptr(rec), _ptr(off), G, _ptr(lam[0]), _ptr(grad_ms), _stream()),
                    "adj_collisions_backward")

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
        st = model.initial_state(m_s)
        checkpoints = []
        for a in range(model.n_adv):
            if a % every == 0:
                checkpoints.append((a, [t.clone() for t in st]))
            model._adv(a, st, k, flux, ni)
        ctx.model, ctx.checkpoints, ctx.k, ctx.s, ctx.ni = model, checkpoints, k, s, ni
        ctx.every = every
        ctx.save_for_backward(m_s, weights)
        return (weights * st[0]).sum()

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
            model.run(kappa=k, flux_scale=s, no_iter=ni, starts=starts, a0=a0, a1=a1,
                      state=state)
            for a in range(a1 - 1, a0 - 1, -1):
                model._adv_bwd(a, starts[a - a0], k, flux, s, ni, lam, grad_ms, grad_k, grad_s)
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
