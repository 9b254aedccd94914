"""Device-resident SIP/grid state and the calls that advance it on the GPU.

``DeviceState`` holds one model state in GPU memory (PyTorch tensors used as
plain device buffers) in the reference's array layout, plus the caller-owned
workspace the C ABI needs.  It is built from the same arrays and scalars the
reference's ``integrate_adv_step_np`` takes (integration.py:1298-1313), runs
advection steps with ``adv_step`` and copies the state back into NumPy arrays
with ``export_to``.

Draw sources for the all-or-nothing collisions:
* ``"philox"``: counter-based Philox4x32-10 on the device, one uniform per
  pair (performance mode);
* ``"thinned"``: the same Philox generator with the thinned draws of
  csrc/lacmo_thin.h: an exact sampler of the same iid per-pair uniforms that
  draws one uniform per low-probability segment of pairs (fastest mode);
* ``"numpy"``: each collision step draws ``np.random.rand(pairs)`` from NumPy's
  global generator on the host, exactly the count and order the reference
  consumes, and copies it to the device (parity mode);
* a 1-D float64 array or CUDA tensor: injected draws consumed in order.
"""
import ctypes

import numpy as np
import torch

from . import _lib
from .constants import solute_code

F64 = torch.float64
_NP_OF = {torch.float64: np.dtype(np.float64), torch.int64: np.dtype(np.int64),
          torch.uint8: np.dtype(np.uint8), torch.int32: np.dtype(np.int32)}

# Philox collision-step counter per seed for the drop-in step functions.  They
# build a fresh device state on every call; without this the counter would
# restart at 0 on each call and every call with the same seed would replay the
# same uniforms, where the reference draws fresh ones each call
# (np.random.rand, collision/all_or_nothing.py:545).
_philox_next = {}


def philox_counter(seed):
    """The collision-step counter the next drop-in call with ``seed`` starts
    from (0 for a seed not used yet in this process)."""
    return _philox_next.get(int(seed), 0)


def reset_philox_counters(seed=None):
    """Restart the drop-in functions' Philox stream of ``seed`` (of every seed
    when None) at collision step 0."""
    if seed is None:
        _philox_next.clear()
    else:
        _philox_next.pop(int(seed), None)


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _copy_to_host(dst, t):
    """Device tensor -> the caller's NumPy array in place: straight into its
    (already resident) pages when dtype and layout allow, else through a
    temporary."""
    if (isinstance(dst, np.ndarray) and dst.flags.c_contiguous and dst.flags.writeable
            and dst.size == t.numel() and torch.from_numpy(dst[:0]).dtype == t.dtype):
        torch.from_numpy(dst).view(-1).copy_(t.reshape(-1))
    else:
        np.copyto(dst, t.cpu().numpy().reshape(np.shape(dst)))


def _upload_into(t, a):
    """The host array ``a`` into the existing device tensor ``t`` (same
    element type and count) in place; False when ``a`` is not such an array
    (a tensor, a scalar, another type or size, a non-contiguous view)."""
    if isinstance(a, torch.Tensor) or np.ndim(a) == 0:
        return False
    arr = np.asarray(a)
    if arr.dtype == np.bool_:
        arr = arr.view(np.uint8)
    if arr.size != t.numel() or not arr.flags.c_contiguous or not arr.flags.writeable:
        return False
    src = torch.from_numpy(arr)
    if src.dtype != t.dtype:
        return False
    t.view(-1).copy_(src.view(-1), non_blocking=True)
    return True


def to_device(a, dtype=F64, device="cuda"):
    """NumPy array / scalar / tensor -> contiguous CUDA tensor of ``dtype``."""
    if isinstance(a, torch.Tensor):
        t = a.to(device=device, dtype=dtype)
        return t.contiguous()
    arr = np.ascontiguousarray(np.asarray(a))
    if not arr.flags.writeable:
        arr = arr.copy()
    t = torch.from_numpy(arr)
    if t.dtype != dtype:
        t = t.to(dtype)
    return t.to(device, non_blocking=False).contiguous()


class DeviceState:
    GRID_KEYS = ("grid_scalar_fields", "grid_mat_prop", "grid_velocity",
                 "grid_mass_flux_air_dry")

    def __init__(self, st, device="cuda", draws="philox", seed=1001, precision="fp64",
                 workspace=True, thin=False, reuse=None):
        """``reuse``: a DeviceState of the same shape (SIP count and grid)
        that is done with: its device buffers (and, for the same parameters
        and draw source, its captured step graph) take this state's data
        instead of new allocations, and it must not be used afterwards."""
        self.lib = _lib.load()
        self.device = device
        g = st["grid_no_cells"]
        self.nx, self.nz = int(g[0]), int(g[1])
        pos = np.asarray(st["pos"]) if not isinstance(st["pos"], torch.Tensor) else st["pos"]
        self.n = int(pos.shape[1])
        self._plan_handle = None
        self._reuse = (reuse if reuse is not None and (reuse.n, reuse.nx, reuse.nz, reuse.device)
                       == (self.n, self.nx, self.nz, device) else None)
        dev = device
        self.pos = self._dev("pos", st["pos"])
        self.vel = self._dev("vel", st["vel"])
        self.rel_pos = self._dev("rel_pos", st["rel_pos"])
        self.m_w = self._dev("m_w", st["m_w"])
        self.m_s = self._dev("m_s", st["m_s"])
        self.xi = self._dev("xi", st["xi"])
        self.T_p = self._dev("T_p", st["T_p"])
        self.water_removed = self._dev("water_removed", st["water_removed"])
        self.no_cols = self._dev("no_cols", st.get("no_cols", np.zeros(2, np.int64)), torch.int64)
        self.cell = (self._reuse.cell if self._reuse is not None
                     else torch.empty(self.n, dtype=torch.int32, device=dev))
        # the reference's cells (int64) and active flags (bool, as bytes)
        self._cells_in = self._dev("_cells_in", st["cells"], torch.int64)
        act = st["active_ids"]
        if not isinstance(act, torch.Tensor):
            act = np.asarray(act)
            act = act.view(np.uint8) if act.dtype == np.bool_ else act.astype(np.uint8)
        self._act_in = self._dev("_act_in", act, torch.uint8)
        s = _stream()
        _lib.check(self.lib.lacmo_cells_import(_ptr(self._cells_in), _ptr(self._act_in),
                                               _ptr(self.cell), self.n, self.nx, self.nz, s),
                   "cells_import")
        self.gsf = self._dev("gsf", st["grid_scalar_fields"])
        self.gmp = self._dev("gmp", st["grid_mat_prop"])
        self.gvel = self._dev("gvel", st["grid_velocity"])
        self.flux = self._dev("flux", st["grid_mass_flux_air_dry"])
        self.delta_m_l = self._dev("delta_m_l", st["delta_m_l"])
        self.grid = self._make_grid(st)
        self.sips = _lib.Sips(self.n, self.pos.data_ptr(), self.vel.data_ptr(),
                              self.rel_pos.data_ptr(), self.m_w.data_ptr(), self.m_s.data_ptr(),
                              self.xi.data_ptr(), self.T_p.data_ptr(), self.cell.data_ptr(),
                              self.water_removed.data_ptr(), self.no_cols.data_ptr())
        if precision not in ("fp64", "mixed"):
            raise ValueError(f"precision must be 'fp64' or 'mixed', got {precision!r}")
        self.precision = precision
        if isinstance(draws, str) and draws == "thinned":
            draws, thin = "philox", True
        self.thin = bool(thin)
        self.set_params(st)
        self.draw_mode = draws if isinstance(draws, str) else "buffer"
        self.seed = int(seed)
        self.draw_buf = None
        if not workspace:   # a batch member: the batch owns the workspace
            self.ws, self.ws_bytes = None, 0
            self._reuse = None
            return
        self.ws_bytes = int(self.lib.lacmo_workspace_bytes(self.n, self.nx, self.nz))
        old = self._reuse
        self.ws = (old.ws if old is not None and old.ws is not None
                   and old.ws_bytes == self.ws_bytes else
                   torch.empty(self.ws_bytes, dtype=torch.uint8, device=dev))
        _lib.check(self.lib.lacmo_workspace_reset(_ptr(self.ws), self.ws_bytes, self.n, self.nx,
                                                  self.nz, s), "workspace_reset")
        if not isinstance(draws, str):
            self.draw_buf = self._dev("draw_buf", draws)
        if old is not None:
            # the captured step graph holds the buffers' addresses, the
            # parameters and the draw source: it carries over when they match
            h = getattr(old, "_plan_handle", None)
            if (h is not None and self.draw_buf is None and old.draw_buf is None
                    and bytes(self.params) == bytes(old.params) and self.seed == old.seed
                    and bytes(self.grid) == bytes(old.grid)
                    and bytes(self.sips) == bytes(old.sips) and self.ws is old.ws):
                self._plan_handle = h
                self._plan_draws = old._plan_draws
                old._plan_handle = None
        self._reuse = None
        self.prepare()

    def _dev(self, name, a, dtype=F64):
        """``a`` on the device: into the reused state's buffer ``name`` when
        it fits, else a new tensor (to_device)."""
        old = getattr(self._reuse, name, None) if getattr(self, "_reuse", None) is not None \
            else None
        if isinstance(old, torch.Tensor) and old.dtype == dtype and _upload_into(old, a):
            return old
        return to_device(a, dtype, self.device)

    # -- parameters -------------------------------------------------------------
    def set_params(self, st):
        dev = self.device
        nz = self.nz
        prof = lambda k, name: (self._dev(name, st[k]) if st.get(k) is not None
                                else torch.zeros(nz, dtype=F64, device=dev))
        self._no_prof = {"prof_rv": st.get("init_profile_r_v") is None,
                         "prof_th": st.get("init_profile_Theta") is None,
                         "t_relax": st.get("relaxation_time_profile") is None}
        self.prof_rv = prof("init_profile_r_v", "prof_rv")
        self.prof_th = prof("init_profile_Theta", "prof_th")
        self.t_relax = prof("relaxation_time_profile", "t_relax")
        E = st["E_col_grid"]
        if isinstance(E, (float, np.floating)) or np.ndim(E) == 0:
            self.E = None
            E_const = float(E)
            nb, lo, bl = 0, 0.0, 1.0
        else:
            self.E = self._dev("E", E)
            E_const = 0.0
            nb, lo, bl = (int(st["no_kernel_bins"]), float(st["R_kernel_low_log"]),
                          float(st["bin_factor_R_log"]))
        self.params = self._make_params(st)

    def _make_params(self, st):
        """The parameter structure of ``st`` over this state's device buffers
        (profiles and efficiency table as set_params placed them)."""
        E = st["E_col_grid"]
        if isinstance(E, (float, np.floating)) or np.ndim(E) == 0:
            E_const, nb, lo, bl = float(E), 0, 0.0, 1.0
        else:
            E_const = 0.0
            nb, lo, bl = (int(st["no_kernel_bins"]), float(st["R_kernel_low_log"]),
                          float(st["bin_factor_R_log"]))
        has_relax = st.get("init_profile_r_v") is not None
        return _lib.Params(
            float(st["dt"]), float(st["dt_sub"]), float(st["dt_sub_half"]),
            float(st["dt_col_over_dV"]), float(st["g_set"]), int(st["scale_dt_cond"]),
            int(st["no_col_per_adv"]), int(bool(st["act_collisions"])),
            int(bool(st["act_relaxation"]) and has_relax), int(st["no_iter_impl_mass"]),
            solute_code(st["solute_type"]), self.prof_rv.data_ptr(), self.prof_th.data_ptr(),
            self.t_relax.data_ptr(), self.E.data_ptr() if self.E is not None else None, E_const,
            nb, lo, bl, _lib.PRECISION_MIXED if getattr(self, "precision", "fp64") == "mixed"
            else _lib.PRECISION_FP64, int(getattr(self, "thin", False)))

    def _make_grid(self, st):
        ranges = np.asarray(st["grid_ranges"], dtype=np.float64)
        steps = np.asarray(st["grid_steps"], dtype=np.float64)
        return _lib.Grid(self.nx, self.nz, self.gsf.data_ptr(), self.gmp.data_ptr(),
                         self.gvel.data_ptr(), self.flux.data_ptr(), self.delta_m_l.data_ptr(),
                         ranges[0, 0], ranges[0, 1], ranges[1, 0], ranges[1, 1], steps[0],
                         steps[1], float(st["grid_volume_cell"]), float(st["p_ref"]),
                         float(st["p_ref_inv"]))

    # host arrays of integrate_adv_step_np and the device buffers they fill
    # (copied in) or take (copied out); cells and active flags go through
    # the import / export kernels
    _IN = (("pos", "pos"), ("vel", "vel"), ("rel_pos", "rel_pos"), ("m_w", "m_w"),
           ("m_s", "m_s"), ("xi", "xi"), ("T_p", "T_p"), ("water_removed", "water_removed"),
           ("no_cols", "no_cols"), ("_cells_in", "cells"), ("_act_in", "active_ids"),
           ("gsf", "grid_scalar_fields"), ("gmp", "grid_mat_prop"), ("gvel", "grid_velocity"),
           ("flux", "grid_mass_flux_air_dry"), ("delta_m_l", "delta_m_l"),
           ("prof_rv", "init_profile_r_v"), ("prof_th", "init_profile_Theta"),
           ("t_relax", "relaxation_time_profile"), ("E", "E_col_grid"))
    _OUT = (("pos", "pos"), ("vel", "vel"), ("rel_pos", "rel_pos"), ("m_w", "m_w"),
            ("m_s", "m_s"), ("xi", "xi"), ("T_p", "T_p"), ("water_removed", "water_removed"),
            ("gsf", "grid_scalar_fields"), ("gmp", "grid_mat_prop"), ("delta_m_l", "delta_m_l"),
            ("no_cols", "no_cols"), ("_cells_out", "cells"), ("_act_out", "active_ids"))

    @staticmethod
    def _host_view(a, t, write):
        """``a`` as a C-contiguous NumPy array of ``t``'s element type and
        count (writeable when ``write``), or None."""
        if not isinstance(a, np.ndarray):
            return None
        if a.dtype == np.bool_:
            a = a.view(np.uint8)
        if (a.size != t.numel() or not a.flags.c_contiguous or (write and not a.flags.writeable)
                or a.dtype != _NP_OF[t.dtype]):
            return None
        return a

    def dropin_step(self, st, seed, draws, precision, col_step=None, copy_mode=None):
        """One integrate_adv_step_np call on the host arrays of ``st`` in one
        native call (lacmo_dropin_adv_step): the arrays are copied into this
        state's buffers, the step replays the captured graph, and the results
        are copied back in place.  Returns False, having done nothing, when
        the call does not fit this state (shape, array types, parameters,
        draw source), for the caller to build a new state instead.
        ``copy_mode``: _lib.COPY_AUTO (None), COPY_ENGINE or COPY_KERNEL (the
        SMs read and write the host pages; where the device can)."""
        thin = draws == "thinned"
        if (self.ws is None or draws not in ("philox", "thinned") or self.draw_mode != "philox"
                or self.thin != thin or self.precision != precision or self.seed != int(seed)
                or self.draw_buf is not None):
            return False
        if getattr(self, "_cells_out", None) is None:
            self._cells_out = torch.empty((2, self.n), dtype=torch.int64, device=self.device)
            self._act_out = torch.empty(self.n, dtype=torch.uint8, device=self.device)
        ins, outs, keep = [], [], []
        for name, key in self._IN:
            t = getattr(self, name)
            a = st.get(key)
            if name in self._no_prof:   # an absent profile stays zeros on the device
                if self._no_prof[name] != (a is None):
                    return False
                if a is None:
                    continue
            elif name == "E":           # a constant efficiency lives in the parameters
                if (t is None) != (np.ndim(a) == 0):
                    return False
                if t is None:
                    continue
            h = self._host_view(a, t, False)
            if h is None:
                return False
            keep.append(h)
            ins.append((t.data_ptr(), h.ctypes.data, h.nbytes))
        for name, key in self._OUT:
            t = getattr(self, name)
            a = st.get(key)
            if a is None:
                continue
            h = self._host_view(a, t, True)
            if h is None:
                return False
            keep.append(h)
            outs.append((h.ctypes.data, t.data_ptr(), h.nbytes))
        if (bytes(self._make_params(st)) != bytes(self.params)
                or bytes(self._make_grid(st)) != bytes(self.grid)):
            return False
        plan = self._plan()
        cin = (_lib.Copy * max(1, len(ins)))(*[_lib.Copy(*e) for e in ins])
        cout = (_lib.Copy * max(1, len(outs)))(*[_lib.Copy(*e) for e in outs])
        d = self._draws_struct()
        after = ctypes.c_int64(0)
        call = _lib.Dropin(cin, len(ins), cout, len(outs), ctypes.pointer(self.sips),
                           ctypes.pointer(self.grid), ctypes.pointer(self.params),
                           ctypes.pointer(d), self.ws.data_ptr(), self.ws_bytes,
                           self._cells_in.data_ptr(), self._act_in.data_ptr(),
                           self._cells_out.data_ptr(), self._act_out.data_ptr(), plan,
                           philox_counter(seed) if col_step is None else int(col_step),
                           ctypes.pointer(after),
                           _lib.COPY_AUTO if copy_mode is None else int(copy_mode))
        _lib.check(self.lib.lacmo_dropin_adv_step(ctypes.byref(call), _stream()), "dropin_adv_step")
        _philox_next[self.seed] = int(after.value)
        return True

    def prepare(self):
        _lib.check(self.lib.lacmo_prepare(ctypes.byref(self.sips), ctypes.byref(self.grid),
                                          ctypes.byref(self.params), _ptr(self.ws), self.ws_bytes,
                                          _stream()), "prepare")

    # -- stepping ---------------------------------------------------------------
    def _draws_struct(self):
        if self.draw_buf is not None:
            return _lib.Draws(self.draw_buf.data_ptr(), self.draw_buf.numel(), self.seed)
        return _lib.Draws(None, 0, self.seed)

    def adv_step(self, n_steps=1, graph=False):
        """``n_steps`` advection steps (integration.py:1298-1611).

        ``graph=True`` replays a CUDA graph of one step (captured on first
        use on a side stream); not available with host-side numpy draws."""
        if self.draw_mode == "numpy":
            for _ in range(n_steps):
                self._adv_step_numpy_draws()
            return
        if graph:
            plan = self._plan()
            s = _stream()
            for _ in range(n_steps):
                _lib.check(self.lib.lacmo_plan_launch(plan, s), "plan_launch")
            return
        d = self._draws_struct()
        s = _stream()
        for _ in range(n_steps):
            _lib.check(self.lib.lacmo_integrate_adv_step(
                ctypes.byref(self.sips), ctypes.byref(self.grid), ctypes.byref(self.params),
                ctypes.byref(d), _ptr(self.ws), self.ws_bytes, s), "integrate_adv_step")

    def _plan(self):
        if getattr(self, "_plan_handle", None) is not None:
            return self._plan_handle
        cur = torch.cuda.current_stream()
        side = torch.cuda.Stream()
        side.wait_stream(cur)
        d = self._draws_struct()
        handle = ctypes.c_void_p()
        with torch.cuda.stream(side):
            _lib.check(self.lib.lacmo_plan_create(
                ctypes.byref(self.sips), ctypes.byref(self.grid), ctypes.byref(self.params),
                ctypes.byref(d), _ptr(self.ws), self.ws_bytes, 1,
                ctypes.c_void_p(side.cuda_stream), ctypes.byref(handle)), "plan_create")
        cur.wait_stream(side)
        self._plan_handle = handle
        self._plan_draws = d
        return handle

    def drop_graph(self):
        """Forget the captured step graph (the next graph step captures a new
        one, e.g. with launch shapes the autotuner changed since)."""
        torch.cuda.synchronize()
        if self._plan_handle is not None:
            self.lib.lacmo_plan_destroy(self._plan_handle)
            self._plan_handle = None

    def retune(self):
        """Time the launch shapes on this batch in its current regime (it
        advances a few steps), set them and drop the captured graph; see
        lacmopy_gb300.autotune.tune_live."""
        from . import autotune
        choice = autotune.tune_live(self)
        self.drop_graph()
        return choice

    def graph_kernel_count(self):
        """Kernel nodes in the captured one-step graph (0 if none)."""
        if getattr(self, "_plan_handle", None) is None:
            return 0
        return int(self.lib.lacmo_plan_kernel_nodes(self._plan_handle))

    def __del__(self):
        h = getattr(self, "_plan_handle", None)
        if h is not None:
            try:
                self.lib.lacmo_plan_destroy(h)
            except Exception:
                pass

    def pair_count(self):
        out = ctypes.c_int64(0)
        _lib.check(self.lib.lacmo_collision_pair_count(_ptr(self.ws), self.n, self.nx, self.nz,
                                                       ctypes.byref(out), _stream()), "pair_count")
        return int(out.value)

    def collision_step(self, draws=None):
        """All-cells collision step (collision/all_or_nothing.py:754-846).

        ``draws``: None uses the state's draw mode; an array/tensor injects."""
        if draws is None and self.draw_mode == "numpy":
            draws = np.random.rand(self.pair_count())
        if draws is not None:
            buf = to_device(draws, device=self.device)
            if buf.numel() == 0:
                buf = torch.zeros(1, dtype=F64, device=self.device)
            d = _lib.Draws(buf.data_ptr(), buf.numel(), self.seed)
        else:
            d = _lib.Draws(None, 0, self.seed)
        _lib.check(self.lib.lacmo_collision_step_cells(
            ctypes.byref(self.sips), ctypes.byref(self.grid), ctypes.byref(self.params),
            ctypes.byref(d), _ptr(self.ws), self.ws_bytes, _stream()), "collision_step_cells")
        torch.cuda.current_stream().synchronize() if draws is not None else None

    def _subloop(self, no_cond, no_col):
        # integration.py:1095-1294
        col = bool(self.params.act_collisions)
        if col and no_col == 1:
            self.collision_step()
        for _ in range(no_cond):
            if col and no_col > 1:
                self.collision_step()
            self._substep(self.params.dt_sub, False)
        if col and no_col > no_cond:
            self.collision_step()

    def _substep(self, dt_pos, write_Tp):
        _lib.check(self.lib.lacmo_adv_substep(
            ctypes.byref(self.sips), ctypes.byref(self.grid), ctypes.byref(self.params),
            float(dt_pos), int(write_Tp), _ptr(self.ws), self.ws_bytes, _stream()), "adv_substep")

    def _adv_step_numpy_draws(self):
        p = self.params
        s = _stream()
        _lib.check(self.lib.lacmo_adv_step_begin(ctypes.byref(self.sips), ctypes.byref(self.grid),
                                                 ctypes.byref(p), _ptr(self.ws), self.ws_bytes, s),
                   "adv_step_begin")
        ncol = p.no_col_per_adv
        self._subloop(p.scale_dt_cond, 0 if ncol == 1 else (1 if ncol == 2 else p.scale_dt_cond))
        _lib.check(self.lib.lacmo_adv_step_second_half(
            ctypes.byref(self.sips), ctypes.byref(self.grid), ctypes.byref(p), _ptr(self.ws),
            self.ws_bytes, s), "adv_step_second_half")
        self._subloop(p.scale_dt_cond - 1, 1 if ncol in (1, 2) else p.scale_dt_cond)
        self._substep(p.dt_sub_half, True)

    def adv_step_tracked(self, record, collide=None):
        """One advection step sub-step by sub-step (integration.py:1474-1610,
        the collision placement of :1095-1294), calling ``record(k)`` before
        particle sub-step k = 0 .. 2 scale_dt_cond - 1, while ``self.cell``
        holds the cells that sub-step's condensation uses, and, for each
        collision step (when the state collides), ``collide(k, step)`` with k
        the next sub-step and ``step`` the function that runs it (default:
        run it)."""
        p = self.params
        s = _stream()
        col = bool(p.act_collisions)
        collide = collide or (lambda k, step: step())
        k = 0

        def subloop(no_cond, no_col):
            nonlocal k
            if col and no_col == 1:
                collide(k, self.collision_step)
            for _ in range(no_cond):
                if col and no_col > 1:
                    collide(k, self.collision_step)
                record(k)
                k += 1
                self._substep(p.dt_sub, False)
            if col and no_col > no_cond:
                collide(k, self.collision_step)

        _lib.check(self.lib.lacmo_adv_step_begin(ctypes.byref(self.sips), ctypes.byref(self.grid),
                                                 ctypes.byref(p), _ptr(self.ws), self.ws_bytes, s),
                   "adv_step_begin")
        ncol = p.no_col_per_adv
        subloop(p.scale_dt_cond, 0 if ncol == 1 else (1 if ncol == 2 else p.scale_dt_cond))
        _lib.check(self.lib.lacmo_adv_step_second_half(
            ctypes.byref(self.sips), ctypes.byref(self.grid), ctypes.byref(p), _ptr(self.ws),
            self.ws_bytes, s), "adv_step_second_half")
        subloop(p.scale_dt_cond - 1, 1 if ncol in (1, 2) else p.scale_dt_cond)
        record(k)
        self._substep(p.dt_sub_half, True)

    def particles_substep(self, dt_sub, dt_sub_pos):
        """integration.py:944 propagate_particles_subloop_step_np."""
        _lib.check(self.lib.lacmo_propagate_particles_subloop_step(
            ctypes.byref(self.sips), ctypes.byref(self.grid), ctypes.byref(self.params),
            float(dt_sub), float(dt_sub_pos), _ptr(self.ws), self.ws_bytes, _stream()),
            "propagate_particles_subloop_step")

    def update_grid_r_l(self):
        _lib.check(self.lib.lacmo_update_grid_r_l(ctypes.byref(self.sips), ctypes.byref(self.grid),
                                                  _ptr(self.ws), self.ws_bytes, _stream()),
                   "update_grid_r_l")

    @property
    def col_step(self):
        """Philox collision-step counter: the step the next collision step
        draws with (synchronises)."""
        v = ctypes.c_int64(0)
        _lib.check(self.lib.lacmo_get_collision_step(_ptr(self.ws), self.n, self.nx, self.nz,
                                                     ctypes.byref(v), _stream()),
                   "get_collision_step")
        return int(v.value)

    @col_step.setter
    def col_step(self, step):
        _lib.check(self.lib.lacmo_set_collision_step(_ptr(self.ws), self.n, self.nx, self.nz,
                                                     int(step), _stream()), "set_collision_step")

    def continue_philox(self, col_step=None):
        """Start this state's Philox draws where the process's previous drop-in
        call with the same seed stopped (or at ``col_step``)."""
        self.col_step = philox_counter(self.seed) if col_step is None else int(col_step)

    def record_philox(self):
        """Remember where this state's Philox draws stopped, for the next
        drop-in call with the same seed."""
        _philox_next[self.seed] = self.col_step

    def fallbacks(self):
        """Mixed precision: SIP sub-steps whose Newton was repeated in FP64."""
        f = ctypes.c_uint64(0)
        _lib.check(self.lib.lacmo_read_fallbacks(_ptr(self.ws), self.n, self.nx, self.nz,
                                                 ctypes.byref(f), _stream()), "read_fallbacks")
        return int(f.value)

    def flags(self):
        f = ctypes.c_uint32(0)
        _lib.check(self.lib.lacmo_read_flags(_ptr(self.ws), self.n, self.nx, self.nz,
                                             ctypes.byref(f), _stream()), "read_flags")
        return int(f.value)

    # -- export -----------------------------------------------------------------
    def cells_and_active(self):
        cells = torch.empty((2, self.n), dtype=torch.int64, device=self.device)
        act = torch.empty(self.n, dtype=torch.uint8, device=self.device)
        g = self.grid
        _lib.check(self.lib.lacmo_cells_export(_ptr(self.cell), _ptr(self.pos), _ptr(self.rel_pos),
                                               _ptr(cells), _ptr(act), self.n, self.nx, self.nz,
                                               g.x_min, g.z_min, g.dx, g.dz, _stream()),
                   "cells_export")
        return cells, act

    def export_to(self, st):
        """Copy the device state into the NumPy arrays of ``st`` in place."""
        cells, act = self.cells_and_active()
        torch.cuda.current_stream().synchronize()
        pairs = [("pos", self.pos), ("vel", self.vel), ("rel_pos", self.rel_pos),
                 ("m_w", self.m_w), ("m_s", self.m_s), ("xi", self.xi), ("T_p", self.T_p),
                 ("water_removed", self.water_removed), ("grid_scalar_fields", self.gsf),
                 ("grid_mat_prop", self.gmp), ("delta_m_l", self.delta_m_l),
                 ("no_cols", self.no_cols), ("cells", cells)]
        for k, t in pairs:
            if k in st and st[k] is not None:
                _copy_to_host(st[k], t)
        if "active_ids" in st and st["active_ids"] is not None:
            dst = st["active_ids"]
            if isinstance(dst, np.ndarray) and dst.dtype == np.bool_ and dst.flags.c_contiguous:
                _copy_to_host(dst.view(np.uint8), act)   # 0/1 bytes are valid booleans
            else:
                np.copyto(dst, act.cpu().numpy().astype(bool))
        return st

    def snapshot(self):
        """The state as a dict of fresh NumPy arrays (reference layout)."""
        cells, act = self.cells_and_active()
        torch.cuda.current_stream().synchronize()
        return {"pos": self.pos.cpu().numpy(), "vel": self.vel.cpu().numpy(),
                "rel_pos": self.rel_pos.cpu().numpy(), "m_w": self.m_w.cpu().numpy(),
                "m_s": self.m_s.cpu().numpy(), "xi": self.xi.cpu().numpy(),
                "T_p": self.T_p.cpu().numpy(), "water_removed": self.water_removed.cpu().numpy(),
                "grid_scalar_fields": self.gsf.cpu().numpy(),
                "grid_mat_prop": self.gmp.cpu().numpy(), "delta_m_l": self.delta_m_l.cpu().numpy(),
                "no_cols": self.no_cols.cpu().numpy(), "cells": cells.cpu().numpy(),
                "active_ids": act.cpu().numpy().astype(bool)}


class BatchState:
    """A batched ensemble: M independent ``DeviceState`` members (same grid
    shape and parameters, own SIP counts and states) advanced together, each
    kernel launch covering every member.  Collision draws come from Philox
    keyed by each member's seed, so member m evolves exactly like a
    ``DeviceState(states[m], draws="thinned", seed=seeds[m])`` on its own
    (``draws="philox"``: per-pair draws).  ``tune=True`` sets the launch
    shapes with the autotuner first (lacmopy_gb300.autotune)."""

    def __init__(self, states, seeds, device="cuda", precision="mixed", draws="thinned",
                 thin=None, tune=False):
        if draws not in ("thinned", "philox"):
            raise ValueError(f"batch draws must be 'thinned' or 'philox', got {draws!r}")
        if thin is None:
            thin = draws == "thinned"
        if len(states) != len(seeds) or not states:
            raise ValueError("one seed per member state is required")
        self.lib = _lib.load()
        if tune:
            # launch shapes timed on a throw-away batch of these states (or
            # taken from the autotuner's cache); see lacmopy_gb300.autotune
            from . import autotune
            autotune.tune_batch(states, seeds, precision=precision, draws=draws)
        self.precision, self.draws = precision, draws
        self.members = [DeviceState(st, device=device, draws="philox", seed=int(sd),
                                    precision=precision, workspace=False, thin=thin)
                        for st, sd in zip(states, seeds)]
        self.M = len(self.members)
        self.params = self.members[0].params
        self.nx, self.nz = self.members[0].nx, self.members[0].nz
        M = self.M
        sips = (_lib.Sips * M)(*[m.sips for m in self.members])
        grids = (_lib.Grid * M)(*[m.grid for m in self.members])
        prms = (_lib.Params * M)(*[m.params for m in self.members])
        seed_arr = (ctypes.c_uint64 * M)(*[m.seed for m in self.members])
        ns = (ctypes.c_int64 * M)(*[m.n for m in self.members])
        self.ws_bytes = int(self.lib.lacmo_batch_workspace_bytes(M, ns, self.nx, self.nz))
        if self.ws_bytes == 0:
            raise _lib.LacmoError("batch_workspace_bytes: invalid member shapes")
        self.ws = torch.empty(self.ws_bytes, dtype=torch.uint8, device=device)
        torch.cuda.current_stream().synchronize()
        h = ctypes.c_void_p()
        _lib.check(self.lib.lacmo_batch_create(M, sips, grids, prms, seed_arr, _ptr(self.ws),
                                               self.ws_bytes, ctypes.byref(h)), "batch_create")
        self.handle = h
        self._keep = (sips, grids, prms, seed_arr, ns)
        self._plan_handle = None
        _lib.check(self.lib.lacmo_batch_prepare(self.handle, ctypes.byref(self.params), _stream()),
                   "batch_prepare")

    @property
    def n_total(self):
        return sum(m.n for m in self.members)

    def adv_step(self, n_steps=1, graph=False):
        s = _stream()
        if graph:
            plan = self._plan()
            for _ in range(n_steps):
                _lib.check(self.lib.lacmo_plan_launch(plan, s), "plan_launch")
            return
        for _ in range(n_steps):
            _lib.check(self.lib.lacmo_batch_adv_step(self.handle, ctypes.byref(self.params), s),
                       "batch_adv_step")

    def _plan(self):
        if self._plan_handle is not None:
            return self._plan_handle
        cur = torch.cuda.current_stream()
        side = torch.cuda.Stream()
        side.wait_stream(cur)
        handle = ctypes.c_void_p()
        with torch.cuda.stream(side):
            _lib.check(self.lib.lacmo_batch_plan_create(
                self.handle, ctypes.byref(self.params), 1, ctypes.c_void_p(side.cuda_stream),
                ctypes.byref(handle)), "batch_plan_create")
        cur.wait_stream(side)
        self._plan_handle = handle
        return handle

    def drop_graph(self):
        """Forget the captured step graph (the next graph step captures a new
        one, e.g. with launch shapes the autotuner changed since)."""
        torch.cuda.synchronize()
        if self._plan_handle is not None:
            self.lib.lacmo_plan_destroy(self._plan_handle)
            self._plan_handle = None

    def retune(self):
        """Time the launch shapes on this batch in its current regime (it
        advances a few steps), set them and drop the captured graph; see
        lacmopy_gb300.autotune.tune_live."""
        from . import autotune
        choice = autotune.tune_live(self)
        self.drop_graph()
        return choice

    def graph_kernel_count(self):
        if self._plan_handle is None:
            return 0
        return int(self.lib.lacmo_plan_kernel_nodes(self._plan_handle))

    def _member_ws(self, m):
        ws, nb = ctypes.c_void_p(), ctypes.c_size_t()
        _lib.check(self.lib.lacmo_batch_member_workspace(self.handle, m, ctypes.byref(ws),
                                                         ctypes.byref(nb)), "member_workspace")
        return ws

    def fallbacks(self, m=None):
        ms = range(self.M) if m is None else [m]
        tot = 0
        for k in ms:
            f = ctypes.c_uint64(0)
            mb = self.members[k]
            _lib.check(self.lib.lacmo_read_fallbacks(self._member_ws(k), mb.n, mb.nx, mb.nz,
                                                     ctypes.byref(f), _stream()), "read_fallbacks")
            tot += int(f.value)
        return tot

    def flags(self, m):
        f = ctypes.c_uint32(0)
        mb = self.members[m]
        _lib.check(self.lib.lacmo_read_flags(self._member_ws(m), mb.n, mb.nx, mb.nz,
                                             ctypes.byref(f), _stream()), "read_flags")
        return int(f.value)

    def snapshot(self, m):
        return self.members[m].snapshot()

    def update_grid_r_l(self, m):
        """grid.py:370 update_grid_r_l_np of member m, with the member's slice
        of the batch workspace (the members are binned by their current cells
        first: a batch step does not bin after its last sub-step)."""
        _lib.check(self.lib.lacmo_batch_rebin(self.handle, _stream()), "batch_rebin")
        ws, nb = ctypes.c_void_p(), ctypes.c_size_t()
        _lib.check(self.lib.lacmo_batch_member_workspace(self.handle, m, ctypes.byref(ws),
                                                         ctypes.byref(nb)), "member_workspace")
        mb = self.members[m]
        _lib.check(self.lib.lacmo_update_grid_r_l(ctypes.byref(mb.sips), ctypes.byref(mb.grid),
                                                  ws, nb.value, _stream()), "update_grid_r_l")

    def __del__(self):
        try:
            if getattr(self, "_plan_handle", None) is not None:
                self.lib.lacmo_plan_destroy(self._plan_handle)
            if getattr(self, "handle", None) is not None:
                self.lib.lacmo_batch_destroy(self.handle)
        except Exception:
            pass
