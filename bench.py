#!/usr/bin/env python3
"""Benchmark of the super-droplet (SIP) hot path on GB300.

One step = one advection step dt = 1 s of the 2-D ICMW 2012 case 1 state:
75 x 75 cells of 20 m, 64 SIPs per cell (~360k SIPs), 10 condensation
sub-steps with the 3-iteration implicit Newton, 2 all-or-nothing collision
steps with the Long/Bott efficiency table, FP64 (the reference's precision).
Synthetic seeded state with the case's shapes and distributions.

Metric: SIP-updates/s = active SIPs advanced one dt per second (whole job).
    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
With N > 1 (torchrun) every rank advances its own independent replica
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

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "SIP-updates/s per timestep on 1 GB300, mixed/batched vs FP64 plain; % HBM roof"
UNIT = "SIP-updates/s"
# algorithmic bytes per SIP of one condensation sub-step (the fused particle
# kernel): reads x, z, u, w, m_w, m_s, xi (8 B each), cell (4 B), flag (1 B)
# = 61 B; writes x, z, u, w, m_w (8 B each) and cell (4 B) = 44 B
BYTES_PARTICLE_SUBSTEP = 105
# per SIP-update (adv step): 53 (half-step move) + 10 * 105 + 2 * 68 (collisions)
BYTES_PER_SIP_UPDATE = 1239


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--nx", type=int, default=75)
    ap.add_argument("--nz", type=int, default=75)
    ap.add_argument("--spcm", type=int, nargs=2, default=[26, 38])
    ap.add_argument("--kernel", default="Long_Bott")
    ap.add_argument("--e2e-steps", type=int, default=3)
    ap.add_argument("--cpu-steps", type=int, default=2)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--precision", default="fp64", choices=["fp64", "mixed"],
                    help="arithmetic of the headline line; the other mode is reported beside it")
    ap.add_argument("--no-graph", action="store_true", help="launch kernels one by one")
    ap.add_argument("--only", action="store_true", help="skip the second precision mode")
    return ap.parse_args()


def workload_config(args, n_sips):
    mode = "fp64_plain" if args.precision == "fp64" else "mixed"
    return {"workload": f"icmw2012_case1_{args.nx}x{args.nz}_{sum(args.spcm)}spc_{mode}",
            "precision_mode": mode, "nx": args.nx, "nz": args.nz,
            "cuda_graph": not getattr(args, "no_graph", False),
            "sips_per_cell": sum(args.spcm), "n_sips": int(n_sips), "kernel": args.kernel,
            "dt_s": 1.0, "cond_substeps": 10, "collision_steps": 2, "newton_iterations": 3,
            "draws": "philox4x32-10 (device)",
            "l2": "flushed between timed steps (512 MiB device memset)",
            "parallelism": "replicas"}


def make_state(args, rank):
    from lacmopy_gb300 import synthetic
    return synthetic.make_icmw_state(Nx=args.nx, Nz=args.nz, no_spcm=tuple(args.spcm),
                                     seed=1001 + rank, kernel_type=args.kernel)


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


# ---------------------------------------------------------------------------
def cpu_port_rate(st, steps, threads):
    """Oracle (C port of the reference path, OpenMP over SIPs and cells) on the
    host cores, Philox draws; returns SIP-updates/s and the seconds spent."""
    from oracle.oracle import Oracle, build
    build()
    orc = Oracle("numba")
    orc.set_threads(threads)
    s = copy.deepcopy(st)
    col_step = np.zeros(1, np.int64)
    n_up = 0
    t0 = time.perf_counter()
    for _ in range(steps):
        n_up += int(np.count_nonzero(s["active_ids"]))
        orc.integrate_adv_step_np(
            s["grid_scalar_fields"], s["grid_mat_prop"], s["grid_velocity"],
            s["grid_mass_flux_air_dry"], s["p_ref"], s["p_ref_inv"], s["grid_no_cells"],
            s["grid_ranges"], s["grid_steps"], s["grid_volume_cell"], s["pos"], s["vel"],
            s["cells"], s["rel_pos"], s["m_w"], s["m_s"], s["xi"], "AS", s["water_removed"], None,
            s["active_ids"], s["T_p"], s["delta_m_l"], s["dt"], s["dt_sub"], s["dt_sub_half"],
            s["dt_col_over_dV"], s["scale_dt_cond"], s["no_col_per_adv"], True, True,
            s["init_profile_r_v"], s["init_profile_Theta"], s["relaxation_time_profile"], 3,
            s["g_set"], s["E_col_grid"], s["no_kernel_bins"], s["R_kernel_low_log"],
            s["bin_factor_R_log"], s["no_cols"], None, None, 1001, col_step)
    dt = time.perf_counter() - t0
    return n_up / dt, dt


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    st = make_state(args, 0)
    threads = os.cpu_count() or 1
    if args.warmup > 0:
        cpu_port_rate(st, min(args.warmup, 1), threads)
    rate, secs = cpu_port_rate(st, args.steps, threads)
    n = int(st["xi"].size)
    line = {"metric": METRIC, "value": rate, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 * secs / args.steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(args, n), "impl": "reference",
            "cpu_baseline": {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"{args.steps} full advection steps of the workload; "
                                       "reference Numba path unavailable on this box (numba "
                                       "not installed), so the C port of the reference "
                                       "algorithm with OpenMP on all host cores"},
            "e2e": {"value": rate, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def run_ours(args):
    import torch
    from lacmopy_gb300 import DeviceState, _lib
    from lacmopy_gb300 import integration as I

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    lib = _lib.load()
    st = make_state(args, rank)
    n = int(st["xi"].size)
    st0 = copy.deepcopy(st)
    flush = torch.empty(512 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    graph = not args.no_graph

    def timed(precision, sample_clocks):
        ds = DeviceState(copy.deepcopy(st), draws="philox", seed=1001 + rank,
                         precision=precision)
        for _ in range(args.warmup):
            ds.adv_step(1, graph=graph)
        torch.cuda.synchronize()
        n_active = []
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        sampler = ClockSampler(local) if sample_clocks else None
        if sampler:
            sampler.start()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        launches0 = lib.lacmo_kernel_launches()
        for k in range(args.steps):
            flush.zero_()
            n_active.append(ds.cell.ge(0).sum())
            ev[k][0].record()
            ds.adv_step(1, graph=graph)
            ev[k][1].record()
        torch.cuda.synchronize()
        launches = lib.lacmo_kernel_launches() - launches0
        if graph:
            # kernels replayed from the captured graph: count them per step
            per_step = ds.graph_kernel_count()
            launches = per_step * args.steps
        clocks = sampler.stop() if sampler else None
        if dist:
            dist.barrier()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        ups = float(sum(int(x) for x in n_active))
        if dist:
            t = torch.tensor([ms], dtype=torch.float64, device="cuda")
            u = torch.tensor([ups], dtype=torch.float64, device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            dist.all_reduce(u, op=dist.ReduceOp.SUM)
            ms, ups = float(t.item()), float(u.item())
        return ds, ms, ups, launches, clocks

    ds, ms, ups, launches, clocks = timed(args.precision, True)
    value = ups / (ms / 1000.0)
    modes = {("fp64_plain" if args.precision == "fp64" else "mixed"):
             {"value": value, "ms_per_step": ms / args.steps}}
    if not args.only:
        other = "mixed" if args.precision == "fp64" else "fp64"
        ds2, ms2, ups2, _, _ = timed(other, False)
        modes["mixed" if other == "mixed" else "fp64_plain"] = {
            "value": ups2 / (ms2 / 1000.0), "ms_per_step": ms2 / args.steps}
        del ds2
    if "mixed" in modes and "fp64_plain" in modes:
        modes["mixed_over_fp64"] = modes["mixed"]["value"] / modes["fp64_plain"]["value"]

    # roofline of the dominant kernel: the fused particle sub-step
    sp, g, p = ds.sips, ds.grid, ds.params
    s = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    kt = []
    for _ in range(10):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        na = int(ds.cell.ge(0).sum())
        a.record()
        _lib.check(lib.lacmo_particles_only(ctypes.byref(sp), ctypes.byref(g), ctypes.byref(p),
                                            p.dt_sub, p.dt_sub, ctypes.c_void_p(ds.ws.data_ptr()),
                                            ds.ws_bytes, s), "particles_only")
        b.record()
        _lib.check(lib.lacmo_bin(ctypes.byref(sp), ctypes.byref(g),
                                 ctypes.c_void_p(ds.ws.data_ptr()), ds.ws_bytes, s), "bin")
        torch.cuda.synchronize()
        kt.append((a.elapsed_time(b), na))
    k_ms = float(np.mean([x[0] for x in kt]))
    k_bytes = BYTES_PARTICLE_SUBSTEP * float(np.mean([x[1] for x in kt]))
    peak, peak_kind = measured_peaks()
    achieved = k_bytes / (k_ms / 1000.0) / 1e9
    roofline = {"bound": "hbm", "kernel": "k_particles (fused condensation/drag/move sub-step)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "peak_source": peak_kind, "traffic": traffic_for("k_particles_icmw75"),
                "kernel_ms": k_ms, "algorithmic_bytes_per_launch": k_bytes,
                "note": "FP64 plain mode is FP64-pipe bound on GB300, not HBM bound"}

    # end to end through the reference-facing API with host NumPy arrays
    e2e = None
    if rank == 0 and args.e2e_steps > 0:
        se = copy.deepcopy(st0)
        keys = I._STATE_KEYS
        h2d = sum(np.asarray(se[k]).nbytes for k in
                  ("pos", "vel", "rel_pos", "m_w", "m_s", "xi", "T_p", "water_removed", "cells",
                   "grid_scalar_fields", "grid_mat_prop", "grid_velocity",
                   "grid_mass_flux_air_dry", "delta_m_l", "init_profile_r_v",
                   "init_profile_Theta", "relaxation_time_profile", "E_col_grid", "no_cols"))
        h2d += n  # active_ids as uint8
        d2h = sum(np.asarray(se[k]).nbytes for k in
                  ("pos", "vel", "rel_pos", "m_w", "m_s", "xi", "T_p", "water_removed", "cells",
                   "grid_scalar_fields", "grid_mat_prop", "delta_m_l", "no_cols")) + n
        I.integrate_adv_step_np(*[se[k] for k in keys], draws="philox", seed=7)  # warm-up
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ups_e = 0
        for _ in range(args.e2e_steps):
            ups_e += int(np.count_nonzero(se["active_ids"]))
            I.integrate_adv_step_np(*[se[k] for k in keys], draws="philox", seed=7)
        torch.cuda.synchronize()
        te = time.perf_counter() - t0
        e2e = {"value": ups_e / te, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h),
               "api": "lacmopy_gb300.integration.integrate_adv_step_np (reference argument "
                      "list, NumPy host arrays copied in and out every call)"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, secs = cpu_port_rate(st0, args.cpu_steps, threads)
        cpu = {"value": rate, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{args.cpu_steps} advection steps of the same {n}-SIP workload, "
                         f"{secs:.1f} s, C port of the reference algorithm, OpenMP"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": workload_config(args, n), "roofline": roofline,
                "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
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
