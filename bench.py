#!/usr/bin/env python3
"""Benchmark of the super-droplet (SIP) hot path on GB300.

Headline workload (the "mixed/batched" side of the metric): an ensemble of 64
independent 2-D ICMW 2012 case 1 states, 75 x 75 cells of 20 m, SIPs per cell
drawn uniformly in [32, 256] per cell and member (~52M SIPs), Hall/Bott
collision efficiencies, mixed precision, Philox collision draws, one advection
step dt = 1 s per step (10 condensation sub-steps with the 3-iteration
implicit Newton, 2 all-or-nothing collision steps), each kernel launch covering
all members, the step replayed from a CUDA graph; thinned Philox draws (an
exact sampler of the per-pair uniforms; the per-pair draws are reported under
"modes").  The headline times fresh states; "modes" also holds the same
ensemble timed after --developed-steps untimed steps, when the cloud rains
and collisions multiply.  The "FP64 plain" side is the single
75 x 75 x 64-SIPs/cell state with the Long/Bott table in FP64, timed with one
Philox uniform per pair and with thinned draws, so that both ratios compare
like with like; both sides and the mixed single state are reported under
"modes".  Seeded synthetic states with the case's shapes and distributions.

Metric: SIP-updates/s = active SIPs advanced one dt per second (whole job).
    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
With N > 1 (torchrun) every rank advances its own independent ensemble
(replicas only; the path needs no collective).
"""
import argparse
import copy
import ctypes
import json
import os
import subprocess
import sys
import threading
import time
from concurrent.futures import ProcessPoolExecutor
import multiprocessing as mp

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "SIP-updates/s per timestep on 1 GB300, mixed/batched vs FP64 plain; % HBM roof"
UNIT = "SIP-updates/s"
# algorithmic bytes per SIP of one condensation sub-step (the fused particle
# kernel): reads x, z, u, w, m_w, m_s, xi (8 B each), cell (4 B), flag (1 B)
# = 61 B; writes x, z, u, w, m_w (8 B each) and cell (4 B) = 44 B.  The
# state stays FP64 in mixed precision, so the figure holds for both modes.
BYTES_PARTICLE_SUBSTEP = 105
# per SIP-update (adv step): 53 (half-step move) + 10 * 105 + 2 * 68 (collisions)
BYTES_PER_SIP_UPDATE = 1239


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--members", type=int, default=64, help="ensemble size of the headline")
    ap.add_argument("--uneven", type=int, nargs=2, default=[32, 256],
                    help="range of SIPs per cell of the ensemble members")
    ap.add_argument("--nx", type=int, default=75)
    ap.add_argument("--nz", type=int, default=75)
    ap.add_argument("--spcm", type=int, nargs=2, default=[26, 38],
                    help="SIPs per cell per aerosol mode of the single-state modes")
    ap.add_argument("--e2e-members", type=int, default=8)
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--cpu-steps", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-single", action="store_true", help="skip the single-state modes")
    ap.add_argument("--no-graph", action="store_true", help="launch kernels one by one")
    ap.add_argument("--draws", default="thinned", choices=["thinned", "philox"],
                    help="collision draws of the headline: thinned Philox draws (an exact "
                         "sampler of the per-pair uniforms) or one Philox uniform per pair")
    ap.add_argument("--no-draws-compare", action="store_true",
                    help="skip the headline ensemble with the other draw mode")
    ap.add_argument("--developed-steps", type=int, default=600,
                    help="untimed steps that advance the headline ensemble to a developed "
                         "(raining) state before the developed-regime timing; 0 skips it")
    ap.add_argument("--no-tune", action="store_true",
                    help="keep the default launch shapes (no autotuning)")
    ap.add_argument("--cpu-1thread-steps", type=int, default=1,
                    help="steps of the single-thread CPU sample (0 skips it)")
    return ap.parse_args()


def workload_config(args):
    """The workload both arms time (the same dict in both JSON lines)."""
    return {"workload": f"icmw2012_case1_{args.nx}x{args.nz}_ensemble{args.members}_"
                        f"uneven{args.uneven[0]}-{args.uneven[1]}spc_hall_bott",
            "members": args.members, "nx": args.nx, "nz": args.nz,
            "sips_per_cell": f"uniform in [{args.uneven[0]}, {args.uneven[1]}] per cell and member",
            "kernel": "Hall_Bott", "dt_s": 1.0, "cond_substeps": 10, "collision_steps": 2,
            "newton_iterations": 3, "regime": "fresh seeded states, advection steps "
                                              f"{args.warmup + 1}-{args.warmup + args.steps}",
            "l2": "inputs larger than L2 (state ~8 GB); L2 also flushed between timed steps "
                  "(512 MiB device memset)",
            "parallelism": "replicas"}


def impl_details(args):
    """How our arm computes the workload (kept out of the shared config)."""
    return {"precision_mode": "mixed",
            "draws": ("philox4x32-10 (device), keyed per member, " +
                      ("thinned draws: one uniform per low-probability segment of pairs, an "
                       "exact sampler of the per-pair uniforms" if args.draws == "thinned"
                       else "one uniform per pair")),
            "cuda_graph": not args.no_graph}


def cpu_model():
    try:
        r = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10)
        for ln in r.stdout.splitlines():
            if ln.split(":")[0].strip() in ("Model name", "Vendor ID"):
                name = ln.split(":", 1)[1].strip()
                if name and ln.startswith("Model name"):
                    return name
    except Exception:
        pass
    import platform
    return platform.processor() or platform.machine()


def numba_probe():
    """Whether the reference's own Numba path can run here."""
    try:
        import numba  # noqa: F401
        return f"numba {numba.__version__} importable"
    except Exception as e:
        return f"numba not importable ({type(e).__name__}: {e})"


def _member_state(a):
    nx, nz, lo, hi, seed = a
    from lacmopy_gb300 import synthetic
    return synthetic.make_icmw_state(Nx=nx, Nz=nz, seed=seed, kernel_type="Hall_Bott",
                                     uneven=(lo, hi))


def make_members(args, rank):
    """The ensemble's states, generated on the host cores in parallel (spawned
    workers: no CUDA context is forked)."""
    jobs = [(args.nx, args.nz, args.uneven[0], args.uneven[1], sd)
            for sd in rank_seeds(rank, args.members)[1]]
    workers = max(1, min(len(jobs), (os.cpu_count() or 1)))
    with ProcessPoolExecutor(workers, mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_member_state, jobs))


def make_single(args, rank):
    from lacmopy_gb300 import synthetic
    return synthetic.make_icmw_state(Nx=args.nx, Nz=args.nz, no_spcm=tuple(args.spcm),
                                     seed=1001 + rank, kernel_type="Long_Bott")


def measured_peaks():
    try:
        with open(os.path.join(REPO, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_for(key):
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as f:
            return json.load(f).get(key)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 7:
                continue
            try:
                sm.append(float(p[0]))
                smax.append(float(p[1]))
            except ValueError:
                continue
            for nm, v in zip(names, p[3:7]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": sorted(reasons),
                "samples": len(sm)}


def aggregate_ranks(ms, ups, dist, device):
    """Whole-job numbers of N replicas: the slowest rank's time and the sum of
    all ranks' SIP updates (value = updates / time)."""
    import torch
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    u = torch.tensor([ups], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def rank_seeds(rank, members):
    """Philox keys and state seeds of a rank's ensemble: disjoint across ranks."""
    return ([1 + 64 * rank + m for m in range(members)],
            [5000 + 1000 * rank + m for m in range(members)])


# ---------------------------------------------------------------------------
def cpu_port_rate(states, steps, threads):
    """Oracle (C port of the reference path, OpenMP over SIPs and cells) on the
    host cores, Philox draws, over the given member states one after another;
    returns SIP-updates/s and the seconds spent."""
    from oracle.oracle import Oracle, build
    build()
    orc = Oracle("numba")
    orc.set_threads(threads)
    n_up = 0
    t0 = time.perf_counter()
    for m, st in enumerate(states):
        s = copy.deepcopy(st)
        col_step = np.zeros(1, np.int64)
        for _ in range(steps):
            n_up += int(np.count_nonzero(s["active_ids"]))
            orc.integrate_adv_step_np(
                s["grid_scalar_fields"], s["grid_mat_prop"], s["grid_velocity"],
                s["grid_mass_flux_air_dry"], s["p_ref"], s["p_ref_inv"], s["grid_no_cells"],
                s["grid_ranges"], s["grid_steps"], s["grid_volume_cell"], s["pos"], s["vel"],
                s["cells"], s["rel_pos"], s["m_w"], s["m_s"], s["xi"], "AS", s["water_removed"],
                None, s["active_ids"], s["T_p"], s["delta_m_l"], s["dt"], s["dt_sub"],
                s["dt_sub_half"], s["dt_col_over_dV"], s["scale_dt_cond"], s["no_col_per_adv"],
                True, True, s["init_profile_r_v"], s["init_profile_Theta"],
                s["relaxation_time_profile"], 3, s["g_set"], s["E_col_grid"],
                s["no_kernel_bins"], s["R_kernel_low_log"], s["bin_factor_R_log"], s["no_cols"],
                None, None, 1 + m, col_step)
    dt = time.perf_counter() - t0
    return n_up / dt, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    from lacmopy_gb300 import synthetic
    # The reference's own path is Numba-compiled Python; without numba it
    # cannot run as shipped, and the C restatement of the reference algorithm
    # (oracle/, FP64, glibc libm, OpenMP over SIPs and cells) runs in its place.
    probe = numba_probe()
    # each step is a bounded sample of the workload: one member (the first
    # member's state) advanced one step, on all host threads
    st = synthetic.make_icmw_state(Nx=args.nx, Nz=args.nz, seed=rank_seeds(0, 1)[1][0],
                                   kernel_type="Hall_Bott", uneven=tuple(args.uneven))
    threads = os.cpu_count() or 1
    if args.warmup > 0:
        cpu_port_rate([st], args.warmup, threads)
    rate, secs = cpu_port_rate([st], args.steps, threads)
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args), "impl": "reference",
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                             "cpu": cpu_model(), "numba_probe": probe,
                             "sample": f"each step: one member ({st['xi'].size} SIPs) of the "
                                       f"{args.members}-member workload advanced one advection "
                                       "step; the reference's Numba path is unavailable (" +
                                       probe + "), so the C restatement of the reference "
                                       "algorithm (FP64, OpenMP over SIPs and cells, one draw "
                                       "per pair) runs"},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    from lacmopy_gb300 import BatchState, DeviceState, _lib
    from lacmopy_gb300 import integration as I

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    members = make_members(args, rank)          # host work before the first CUDA call
    single = None if args.no_single else make_single(args, rank)
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib = _lib.load()
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    graph = not args.no_graph
    peak, peak_kind = measured_peaks()

    def timed(obj, sample_clocks):
        for _ in range(args.warmup):
            obj.adv_step(1, graph=graph)
        torch.cuda.synchronize()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        cells = [m.cell for m in obj.members] if isinstance(obj, BatchState) else [obj.cell]
        n_active = []
        sampler = ClockSampler(local) if sample_clocks else None
        if sampler:
            sampler.start()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        launches0 = lib.lacmo_kernel_launches()
        for k in range(args.steps):
            flush.zero_()
            n_active.append(sum(c.ge(0).sum() for c in cells))
            ev[k][0].record()
            obj.adv_step(1, graph=graph)
            ev[k][1].record()
        torch.cuda.synchronize()
        launches = lib.lacmo_kernel_launches() - launches0
        if graph:
            # kernels replayed from the captured graph: count them per step
            launches = obj.graph_kernel_count() * args.steps
        clocks = sampler.stop() if sampler else None
        if dist:
            dist.barrier()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        ups = float(sum(int(x) for x in n_active))
        if dist:
            ms, ups = aggregate_ranks(ms, ups, dist, "cuda")
        return ms, ups, launches, clocks

    # ---- headline: the batched mixed-precision ensemble ----
    seeds = rank_seeds(rank, args.members)[0]
    t_tune = time.perf_counter()
    batch = BatchState(members, seeds, precision="mixed", draws=args.draws,   # copies to the GPU
                       tune=not args.no_tune)
    tune_s = time.perf_counter() - t_tune
    from lacmopy_gb300 import autotune
    shapes = autotune.current()
    n_total = batch.n_total
    ms, ups, launches, clocks = timed(batch, True)
    value = ups / (ms / 1000.0)
    modes = {"batched_mixed": {"value": value, "ms_per_step": ms / args.steps,
                               "n_sips": n_total, "members": args.members}}

    # roofline of the dominant kernel: the fused mixed particle sub-step over
    # all members (one launch; state advanced afterwards is not used)
    p = batch.params
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    kt = []
    n_act = float(sum(int(m.cell.ge(0).sum()) for m in batch.members))
    for _ in range(5):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        _lib.check(lib.lacmo_batch_particles_only(batch.handle, ctypes.byref(p), s),
                   "batch_particles_only")
        b.record()
        torch.cuda.synchronize()
        kt.append(a.elapsed_time(b))
    k_ms = float(np.mean(kt))
    k_bytes = BYTES_PARTICLE_SUBSTEP * n_act
    achieved = k_bytes / (k_ms / 1000.0) / 1e9
    tr = traffic_for("k_particles_mixed_batch_per_sip")
    roofline = {"bound": "hbm", "kernel": "k_particles_mixed (fused condensation/drag/move "
                                          "sub-step, all members in one launch)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind,
                "traffic": (tr * n_act if tr is not None else None),
                "kernel_ms": k_ms, "algorithmic_bytes_per_launch": k_bytes,
                "bytes_per_sip": BYTES_PARTICLE_SUBSTEP}
    del batch
    torch.cuda.empty_cache()
    modes[f"batched_mixed_{args.draws}_draws"] = {"value": value, "ms_per_step": ms / args.steps}
    if not args.no_draws_compare:
        other = "philox" if args.draws == "thinned" else "thinned"
        batch = BatchState(members, seeds, precision="mixed", draws=other)
        ms_o, ups_o, _, _ = timed(batch, False)
        modes[f"batched_mixed_{other}_draws"] = {"value": ups_o / (ms_o / 1000.0),
                                                  "ms_per_step": ms_o / args.steps}
        del batch
        torch.cuda.empty_cache()

    # ---- the developed regime: the same ensemble advanced (untimed) until
    # the cloud rains, then timed the same way ----
    if args.developed_steps > 0:
        batch = BatchState(members, seeds, precision="mixed", draws=args.draws)
        t0 = time.perf_counter()
        for _ in range(args.developed_steps):
            batch.adv_step(1, graph=graph)
        torch.cuda.synchronize()
        spin_s = time.perf_counter() - t0
        shapes_d = batch.retune() if not args.no_tune else autotune.current()
        cols = sum(int(m.no_cols.sum()) for m in batch.members)
        ms_d, ups_d, _, _ = timed(batch, False)
        cols_d = sum(int(m.no_cols.sum()) for m in batch.members) - cols
        modes["batched_mixed_developed"] = {
            "value": ups_d / (ms_d / 1000.0), "ms_per_step": ms_d / args.steps,
            "regime": f"after {args.developed_steps} untimed advection steps "
                      f"({args.developed_steps} s of model time, {spin_s:.0f} s of wall time) "
                      f"of the headline ensemble, then {args.warmup} warm-up and "
                      f"{args.steps} timed steps",
            "collisions_per_step": cols_d / (args.warmup + args.steps),
            "launch_shapes": shapes_d,
            "over_fresh": (ups_d / (ms_d / 1000.0)) / value}
        del batch
        torch.cuda.empty_cache()
        autotune.apply(shapes)   # the headline's shapes for the modes below

    # ---- the FP64 plain path and the mixed single state (75 x 75 x 64) ----
    if single is not None:
        for prec, dr, key in (("fp64", "philox", "fp64_plain"),
                              ("fp64", "thinned", "fp64_plain_thinned"),
                              ("mixed", "philox", "mixed_single")):
            ds = DeviceState(copy.deepcopy(single), draws=dr, seed=1001 + rank,
                             precision=prec)
            ms2, ups2, _, _ = timed(ds, False)
            modes[key] = {"value": ups2 / (ms2 / 1000.0), "ms_per_step": ms2 / args.steps,
                          "n_sips": int(single["xi"].size), "draws": dr,
                          "workload": f"icmw2012_case1_{args.nx}x{args.nz}_{sum(args.spcm)}spc_"
                                      f"long_bott_{prec}"}
            del ds
        fp = modes["fp64_plain"]["value"]
        fpt = modes["fp64_plain_thinned"]["value"]
        modes["batched_mixed_over_fp64_plain"] = value / fp
        modes["ratio_thinned_over_thinned"] = modes["batched_mixed_thinned_draws"]["value"] / fpt
        if "batched_mixed_philox_draws" in modes:
            modes["ratio_per_pair_over_per_pair"] = (
                modes["batched_mixed_philox_draws"]["value"] / fp)
        modes["mixed_single_over_fp64_plain"] = modes["mixed_single"]["value"] / fp

    # ---- end to end through the reference-facing drop-in API: each member's
    # NumPy state copied in and out by integrate_adv_step_np every step ----
    e2e = None
    if rank == 0 and args.e2e_steps > 0 and args.e2e_members > 0:
        keys = I._STATE_KEYS
        sts = [copy.deepcopy(members[m]) for m in range(min(args.e2e_members, args.members))]
        h2d = d2h = 0
        for se in sts:
            n = int(se["xi"].size)
            h2d += sum(np.asarray(se[k]).nbytes for k in
                       ("pos", "vel", "rel_pos", "m_w", "m_s", "xi", "T_p", "water_removed",
                        "cells", "grid_scalar_fields", "grid_mat_prop", "grid_velocity",
                        "grid_mass_flux_air_dry", "delta_m_l", "init_profile_r_v",
                        "init_profile_Theta", "relaxation_time_profile", "E_col_grid",
                        "no_cols")) + n
            d2h += sum(np.asarray(se[k]).nbytes for k in
                       ("pos", "vel", "rel_pos", "m_w", "m_s", "xi", "T_p", "water_removed",
                        "cells", "grid_scalar_fields", "grid_mat_prop", "delta_m_l",
                        "no_cols")) + n
        import threading

        updates = [0] * len(sts)   # SIP updates of the calls, per member

        def calls(m, n_calls, bar=None, errs=None):
            se = sts[m]
            try:
                with torch.cuda.stream(streams[m]):
                    if bar is not None:
                        bar.wait()
                    for _ in range(n_calls):
                        updates[m] += int(np.count_nonzero(se["active_ids"]))
                        I.integrate_adv_step_np(*[se[k] for k in keys], draws=args.draws,
                                                seed=7 + m, precision="mixed")
                    torch.cuda.current_stream().synchronize()
            except BaseException as ex:   # re-raised by the main thread
                if errs is not None:
                    errs.append(ex)
                raise

        def threaded(n_calls):
            bar, errs = threading.Barrier(len(sts) + 1), []
            ths = [threading.Thread(target=calls, args=(m, n_calls, bar, errs))
                   for m in range(len(sts))]
            for th in ths:
                th.start()
            bar.wait()
            t0 = time.perf_counter()
            for th in ths:
                th.join()
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
            if errs:
                raise errs[0]
            return t

        streams = [torch.cuda.Stream() for _ in sts]
        threaded(1)   # warm-up: one call per member (device buffers, step graph)
        # one host thread and CUDA stream per member, calls overlapping
        updates[:] = [0] * len(sts)
        te = threaded(args.e2e_steps)
        ups_e = sum(updates)
        # the same calls one after another from one thread
        updates[:] = [0] * len(sts)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            for m in range(len(sts)):
                calls(m, 1)
        torch.cuda.synchronize()
        ts = time.perf_counter() - t0
        ups_s = sum(updates)
        e2e = {"value": ups_e / te, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h),
               "api": "lacmopy_gb300.integration.integrate_adv_step_np (reference argument "
                      "list, precision=\"mixed\") per member and step, NumPy host state "
                      "copied in and out every call (into the device buffers and step graph "
                      "the previous call of the same shape left; one untimed call per member "
                      "first); one host thread and CUDA stream per member, calls overlapping",
               "sample": f"{len(sts)} members x {args.e2e_steps} steps of the workload",
               "sequential": {"value": ups_s / ts, "unit": UNIT,
                              "api": "the same calls one after another from one thread"}}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, secs = cpu_port_rate(members[:1], args.cpu_steps, threads)
        probe = numba_probe()
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "cpu": cpu_model(), "numba_probe": probe,
               "sample": f"{args.cpu_steps} advection step(s) of one ensemble member "
                         f"({members[0]['xi'].size} SIPs), {secs:.1f} s; C restatement of "
                         "the reference algorithm in FP64, OpenMP on all host cores (the "
                         "reference's Numba path is unavailable: " + probe + ")"}
        if args.cpu_1thread_steps > 0:
            rate1, secs1 = cpu_port_rate(members[:1], args.cpu_1thread_steps, 1)
            cpu["single_thread"] = {"value": rate1, "unit": UNIT, "cores": 1,
                                    "sample": f"{args.cpu_1thread_steps} advection step(s) of "
                                              f"the same member, {secs1:.1f} s, one thread"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "mixed f32/f64 (f32 Newton, drag and pair screen; f64 state, "
                         "per-cell sums, near-critical Newton and collision updates)",
                "data": "synthetic", "config": workload_config(args),
                "impl_details": dict(impl_details(args), n_sips=int(n_total),
                                     launch_shapes=shapes,
                                     autotune=("off" if args.no_tune else
                                               f"timed on a throw-away batch of the members "
                                               f"({tune_s:.1f} s incl. the batch upload)")),
                "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
                "gpu_launches": int(launches), "modes": modes,
                "hbm_frac_whole_step": value * BYTES_PER_SIP_UPDATE / 1e9 / peak}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_ours(a)
