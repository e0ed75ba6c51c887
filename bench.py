#!/usr/bin/env python3
"""RKHEVI step throughput on GB300.

Workload: GAME's RKHEVI dynamical-core step at RES_ID=6 (40962 cells, 122880
edges), 26 layers, moist build (6 constituents), flat, the baroclinic jet of
Jablonowski and Williamson (2006) with 70 % relative humidity below 8 km and
N(0, 0.5 m/s) wind noise (synthetic, seeded), dt = 100 s.  A "step"
is one pass of the reference's time loop (src/coordinator.c:302-324):
linear_combine_two_states(new -> old) followed by manage_rkhevi, both through
the library's C ABI.

value     mixed-precision step (FP32 horizontal operators, vertical
          eliminations in double-float, FP64 state and tendencies),
          device-resident, steps/s, CUDA events on the library's stream; the
          FP64 step and the mixed step with FP64 eliminations beside it.
e2e       the same loop in the default host-in/host-out mode: every call
          copies its State arguments from pinned host memory to the device and
          its results back, as a reference driver linked against the library
          would run it.
roofline  dominant kernel of the step: algorithmic bytes per launch / its mean
          launch time (events around every kernel in a separate profiled pass
          of the same steps), against the measured HBM copy bandwidth.
cpu_baseline  the oracle (C restatement of the reference, OpenMP over the same
          loops as the reference) on this host's cores, bounded sample.

--impl reference runs the CPU implementation of the same workload (the
oracle port, all host threads) and prints the same metric.  Under torchrun
(N > 1) every rank runs an independent replica (the path does not shard
without a halo exchange, which the reference does not have); value is the
total over ranks.
"""
import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "RKHEVI steps/s at RES_ID=6 L26: FP32-mixed vs FP64 GPU; adjoint/forward cost"
L = 26


# ------------------------------------------------------------------ sizes
def grid_sizes(res, nl=L):
    p4 = 4 ** res
    nc, ne, nt = 10 * p4 + 2, 30 * p4, 20 * p4
    s = nl * nc
    vt = nl * ne + (nl + 1) * nc
    dv = (nl + 1) * ne + nl * nt
    return dict(nc=nc, ne=ne, nt=nt, s=s, vt=vt, dv=dv, nl=nl)


def b_step(res, n_const, w_s, w_t, w_g, nl=L):
    """Compulsory bytes of one RKHEVI step: every state, tendency and grid
    array touched once per substage, B = 2 [3 B_state + 2 B_tend + B_grid]."""
    g = grid_sizes(res, nl)
    b_state = ((n_const + 3) * g["s"] + g["vt"]) * w_s
    b_tend = ((n_const + 1) * g["s"] + nl * g["ne"]) * w_t
    b_grid = (6 * g["vt"] + 12 * g["s"] + 16 * g["ne"] + 2 * g["dv"]) * w_g \
        + (26 * g["ne"] + 12 * g["nc"] + 6 * g["nt"]) * 4
    return 2 * (3 * b_state + 2 * b_tend + b_grid)


def kernel_bytes(res, n_const, r, nl=L):
    """Algorithmic bytes of one non-first step's launches of each kernel of
    the mixed path: every array a kernel reads or writes, counted once per
    launch (r = bytes of the horizontal type and of the FP32 state shadow,
    FP64 state / tendencies / solver work 8, indices 4).  The extra terrain
    terms of the orography layers are left out, so these are lower bounds.
    Returns name -> (bytes per step, launches per step)."""
    g = grid_sizes(res, nl)
    nc, ne, nt, s = g["nc"], g["ne"], g["nt"], g["s"]
    wl, ul, zl, tl = (nl + 1) * nc, nl * ne, (nl + 1) * ne, nl * nt
    wi = (nl - 1) * nc          # inner interfaces
    d, i = 8, 4
    C = n_const
    moist = C > 1
    out = {}
    out["k_make_shadow"] = (((C + 3) * s + wl + ul) * (d + r), 1)
    out["k_cell_prepare"] = (((C + 4) * s + 9 * s) * d + 2 * s * r if moist else 5 * s * d, 1)
    # rk 1 only (advection recomputed in the second substage)
    out["k_tri_vort"] = (3 * ul * r + 6 * nt * i + 3 * tl * r, 1)
    out["k_edge_vort"] = ((ul + wl + s) * r + tl * r + 4 * ne * i + zl * r + ul * r + wl * r + 6 * ne * r
                          + 4 * ne * (r + i) + tl * r + zl * r + 2 * ul * r, 1)
    out["k_cell_kinetic"] = ((ul + wl + s) * r + 8 * s * r + 6 * nc * i + s * r + wl * r, 1)
    # first substage: the pressure gradient gathers one float4 of cell
    # factors per cell (k_pg_cells)
    out["k_pg_cells"] = ((C + 3) * s * r + 4 * s * r, 1)
    rk0_h = 4 * s * r + 3 * ul * r + 2 * ne * i + 3 * ul * r + 2 * ul * r + 3 * ul * d + ul * r
    rk1_h = (2 * ul + zl) * r + 10 * ne * (r + 2 * i) + 2 * ne * i + 2 * s * r + wl * r + s * r + ul * r \
        + 4 * ul * r + 2 * ul * d + ul * d + ul * d + ul * r
    out["k_momentum_h"] = (rk0_h + rk1_h, 2)
    rk0_v = 4 * s * r + 2 * wl * r + wl * r + 2 * wl * r + wl * r + wl * d
    rk1_v = 6 * nc * i + 6 * s * r + ul * r + zl * r + 4 * wl * r + s * r + C * s * r + wl * r + 2 * wl * d
    out["k_momentum_v"] = (rk0_v + rk1_v, 2)
    out["k_theta"] = (2 * 3 * s * r, 2)
    sc = C * s * r + s * r + 2 * ul * r + 18 * nc * i + s * d + wl * r + (C + 1) * s * d
    if moist:
        sc += 7 * s * d + 4 * s * r
    out["k_scalar_tend"] = (2 * sc + (C + 1) * s * d, 2)
    out["k_waves_layer"] = ((11 + 12 + 16) * s * d, 2)
    out["k_waves_rows"] = (2 * (14 * wi + 8 * s) * d, 2)
    out["k_waves_thomas"] = (2 * 6 * wi * d, 2)
    out["k_waves_apply"] = (2 * ((4 * wi + 12 * s + 2 * wl) * d + (4 * s + wi) * r), 2)
    if moist:
        out["k_tracers_solve"] = (2 * ((3 * (C - 1) * s + 3 * wl + s) * d + (C - 1) * s * r), 2)
        out["k_tracers_sedheat"] = ((((C - 2) + 5) * s + 2 * wl) * d, 1)
    return out


PROFILE_JSON = os.path.join(ROOT, "profiles", "ncu_rkhevi_res6_mixed.json")


# ncu raw-page metrics kept per kernel in the machine-written summary
NCU_METRICS = {
    "gpu__time_duration.sum": "duration_ns",
    "dram__bytes_read.sum": "dram_read_bytes",
    "dram__bytes_write.sum": "dram_write_bytes",
    "gpu__dram_throughput.avg.pct_of_peak_sustained_elapsed": "dram_throughput_pct",
    "sm__inst_executed_pipe_fp64.avg.pct_of_peak_sustained_active": "fp64_pipe_pct",
    "sm__pipe_fma_cycles_active.avg.pct_of_peak_sustained_active": "fma_pipe_pct",
    "sm__pipe_alu_cycles_active.avg.pct_of_peak_sustained_active": "alu_pipe_pct",
    "sm__inst_executed_pipe_xu.avg.pct_of_peak_sustained_active": "xu_pipe_pct",
    "sm__warps_active.avg.pct_of_peak_sustained_active": "warps_active_pct",
    "sm__throughput.avg.pct_of_peak_sustained_elapsed": "sm_throughput_pct",
    "launch__registers_per_thread": "registers_per_thread",
    "smsp__inst_executed.sum": "warp_instructions",
    "lts__t_sector_hit_rate.pct": "l2_hit_pct",
    "l1tex__t_sector_hit_rate.pct": "l1_hit_pct",
    "smsp__warp_issue_stalled_long_scoreboard_per_warp_active.pct": "stall_long_scoreboard_pct",
    "smsp__warp_issue_stalled_no_instruction_per_warp_active.pct": "stall_no_instruction_pct",
    "smsp__warp_issue_stalled_lg_throttle_per_warp_active.pct": "stall_lg_throttle_pct",
    "smsp__warp_issue_stalled_math_pipe_throttle_per_warp_active.pct": "stall_math_pipe_throttle_pct",
    "smsp__warp_issue_stalled_wait_per_warp_active.pct": "stall_wait_pct",
    "smsp__warp_issue_stalled_short_scoreboard_per_warp_active.pct": "stall_short_scoreboard_pct",
}


# ncu's units (second row of a raw-page CSV) -> the summary's: nanoseconds
# and bytes
NCU_UNIT_SCALE = {"nsecond": 1.0, "ns": 1.0, "usecond": 1e3, "us": 1e3, "msecond": 1e6, "ms": 1e6, "second": 1e9,
                  "byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9, "KB": 1e3, "MB": 1e6, "GB": 1e9}


# the step's timing scopes (game_gpu_profile names) -> the kernels ncu sees
# under them on the mixed path, double-float eliminations first
NCU_NAMES = {
    "k_scalar_tend": ("k_scalar_tend2",),
    "k_waves_layer": ("k_waves_layer_df", "k_waves_layer"),
    "k_waves_rows": ("k_waves_rows_df", "k_waves_rows_mixed"),
    "k_waves_thomas": ("k_waves_thomas_df", "k_waves_thomas"),
    "k_waves_apply": ("k_waves_apply_df", "k_waves_apply"),
    "k_tracers_solve": ("k_tracers_solve_df", "k_tracers_solve"),
    "k_tracers_sedheat": ("k_tracers_sedheat_df", "k_tracers_sedheat"),
    "k_cell_prepare": ("k_cell_prepare_f32", "k_cell_prepare"),
}


def short_kernel_name(full):
    """'void game::<anon>::k_waves_df<26>(...)' -> 'k_waves_df'"""
    import re
    for name in re.findall(r"([A-Za-z_]\w*)\s*[<(]", full):
        if name != "void":
            return name
    return full.strip()


def ncu_json(args):
    """--ncu-json RAW.csv [RAW.csv ...]: summarise `ncu -i REPORT --page raw
    --csv` outputs per kernel (launches; means per launch of the metrics in
    NCU_METRICS) into --out, with the commit of this checkout and the capture
    command"""
    import csv
    kernels = {}
    for path in args.ncu_json:
        with open(path) as f:
            rows = list(csv.reader(f))
        if not rows:
            continue
        head, units = rows[0], rows[1]
        data = [r for r in rows[2:] if len(r) == len(head)]
        col = {n: i for i, n in enumerate(head)}
        for r in data:
            name = short_kernel_name(r[col["Kernel Name"]])
            k = kernels.setdefault(name, {"launches": 0, "sums": {}})
            k["launches"] += 1
            for metric, key in NCU_METRICS.items():
                if metric in col:
                    try:
                        v = float(r[col[metric]].replace(",", ""))
                    except ValueError:
                        continue
                    k["sums"][key] = k["sums"].get(key, 0.0) + v * NCU_UNIT_SCALE.get(units[col[metric]].strip(), 1.0)
    out = {}
    for name, k in kernels.items():
        e = {"launches": k["launches"]}
        for key, v in k["sums"].items():
            e[key] = v / k["launches"]
        if "dram_read_bytes" in e and "dram_write_bytes" in e:
            e["dram_bytes_per_launch"] = e["dram_read_bytes"] + e["dram_write_bytes"]
        out[name] = e
    try:
        commit = subprocess.run(["git", "-C", ROOT, "rev-parse", "HEAD"], capture_output=True, text=True,
                                timeout=30).stdout.strip() or None
    except (OSError, subprocess.TimeoutExpired):
        commit = None
    summary = {"commit": commit, "captured": args.captured, "command": args.command, "kernels": out}
    with open(args.out, "w") as f:
        json.dump(summary, f, indent=1, sort_keys=True)
        f.write("\n")


def read_profile(kernel, key):
    """(value, source) of a per-kernel figure from the machine-written ncu
    summary (written by --ncu-json from an ncu capture; it records the commit
    the capture ran at), or (None, None)"""
    try:
        with open(PROFILE_JSON) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None, None
    kernels = d.get("kernels", {})
    k = None
    for name in NCU_NAMES.get(kernel, (kernel,)):
        if name in kernels and key in kernels[name]:
            k = kernels[name]
            break
    if k is None:
        return None, None
    return k[key], {"file": os.path.relpath(PROFILE_JSON, ROOT), "commit": d.get("commit"),
                    "captured": d.get("captured")}


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during a region"""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    sm.append(float(parts[1]))
                    mx.append(float(parts[2]))
                except ValueError:
                    continue
                for n, v in zip(names, parts[5:9]):
                    if v.lower() == "active":
                        reasons.add(n)
        os.unlink(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "samples": len(sm),
                "reasons": sorted(reasons)}


# ------------------------------------------------------------------ set-up
MOUNTAIN = (2000.0, 1.5e6, 30.0, 90.0)   # 2 km Gaussian mountain, 1500 km half-width, 30N 90E


def build_model(res, moist, n_lloyd, pinned, mountain=None, n_layers=L):
    """grid tables from the input cache (built on first use), host structs"""
    from game_archived_gb300 import abi, cases, structs, tables, workloads
    tab = tables.cached(workloads.input_dir(), res, n_layers=n_layers, n_lloyd=n_lloyd, mountain=mountain)
    lay = structs.Layout(res, n_layers, moist)
    m = abi.pinned_model(lay) if pinned else structs.Model(lay)
    tables.fill_grid(tab, m.grid, m.dualgrid)
    cases.default_config(m)
    return tab, m


def copy_model(src, pinned):
    from game_archived_gb300 import abi, structs
    m = abi.pinned_model(src.layout) if pinned else structs.Model(src.layout)
    for k in structs.Model.KINDS:
        getattr(m, k).copy_from(getattr(src, k))
    return m


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


# ------------------------------------------------------------------ GPU arm
def device_used_bytes(device):
    """bytes in use on the device (cudaMemGetInfo: total - free)"""
    import torch
    free, total = torch.cuda.mem_get_info(device)
    return total - free


def repeats_for(ms_per_step, steps, min_seconds):
    """how many blocks of `steps` steps make a timed region of at least
    min_seconds"""
    if min_seconds <= 0 or ms_per_step <= 0:
        return 1
    return max(1, math.ceil(min_seconds * 1e3 / (ms_per_step * steps)))


def time_resident(model0, precision, steps, warmup, dt, device, sampler=None, profile=False, column_solver=0,
                  mem_used=None, min_seconds=0.0, double_float=1, world=1, info=None):
    """ms per step of the device-resident step; the timed region runs
    `steps` steps, repeated until it covers min_seconds (the estimate comes
    from a few untimed steps after the warm-up), between two barriers and
    synchronisations; info receives the number of timed steps"""
    from game_archived_gb300 import abi, driver
    m = copy_model(model0, pinned=False)
    g = abi.GpuModel(m, precision, resident=True, graphs=True, device=device, column_solver=column_solver,
                     double_float=double_float)
    try:
        for s in (m.state_old, m.state_new, m.state_tendency):
            g.sync_to_device(s)
        driver.start(m, g.linear_combine_two_states)
        t = 0.0
        for n in range(warmup):
            driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, dt, t)
            t += dt
        g.synchronize()
        g.event_record(0)
        for n in range(3):
            driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, dt, t)
            t += dt
        g.event_record(1)
        g.synchronize()
        est = allreduce_max(g.event_elapsed_ms(0, 1) / 3, world)
        n_timed = steps * repeats_for(est, steps, min_seconds)
        g.kernel_launches(reset=True)
        barrier(world)
        g.synchronize()
        if sampler:
            sampler.start()
        g.event_record(0)
        for n in range(n_timed):
            driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, dt, t)
            t += dt
        g.event_record(1)
        g.synchronize()
        barrier(world)
        ms = g.event_elapsed_ms(0, 1)
        clocks = sampler.stop() if sampler else None
        launches = g.kernel_launches()
        if info is not None:
            info["timed_steps"] = n_timed
            info["launches_per_step"] = launches / n_timed
        prof = None
        if profile:
            g.profile(True)
            for n in range(steps):
                driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, dt, t)
                t += dt
            g.profile(False)
            prof = g.profile_results()
        g.sync_to_host(m.state_new)
        if mem_used is not None:
            mem_used.append(device_used_bytes(device))
        import numpy as np
        finite = bool(np.isfinite(m.state_new["rho"]).all() and np.isfinite(m.state_new["wind"]).all())
        return ms / n_timed, launches, clocks, prof, finite
    finally:
        g.close()


def time_e2e(model0, precision, steps, warmup, dt, device, min_seconds=0.0, world=1, info=None):
    """seconds per step of the reference's time loop through the C ABI in the
    default host-in/host-out mode (pinned host structs): every step copies
    its State arguments in and its results out.  Repeated like
    time_resident until the timed region covers min_seconds."""
    from game_archived_gb300 import abi, driver
    m = copy_model(model0, pinned=True)
    g = abi.GpuModel(m, precision, resident=False, graphs=True, device=device)
    try:
        driver.start(m, g.linear_combine_two_states)
        t = 0.0
        for n in range(warmup):
            driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, dt, t)
            t += dt
        g.synchronize()
        t0 = time.perf_counter()
        for n in range(2):
            driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, dt, t)
            t += dt
        g.synchronize()
        est = allreduce_max((time.perf_counter() - t0) * 1e3 / 2, world)
        n_timed = steps * repeats_for(est, steps, min_seconds)
        g.transfer_bytes(reset=True)
        barrier(world)
        t0 = time.perf_counter()
        for n in range(n_timed):
            driver.step(m, g.linear_combine_two_states, g.manage_rkhevi, dt, t)
            t += dt
        g.synchronize()
        sec = time.perf_counter() - t0
        barrier(world)
        h2d, d2h = g.transfer_bytes()
        if info is not None:
            info["timed_steps"] = n_timed
        return sec / n_timed, h2d // n_timed, d2h // n_timed
    finally:
        g.close()


def cap_weights(m, lat0=45.0, lon0=0.0, radius_deg=20.0):
    """area_sfc of the columns within radius_deg of (lat0, lon0), else 0"""
    import numpy as np
    lay = m.layout
    lat, lon = m.grid["latitude_scalar"][:lay.nc], m.grid["longitude_scalar"][:lay.nc]
    p0, l0 = np.radians(lat0), np.radians(lon0)
    cosd = np.sin(lat) * np.sin(p0) + np.cos(lat) * np.cos(p0) * np.cos(lon - l0)
    area_sfc = m.grid["area"][lay.n_vectors - lay.nc:lay.n_vectors]
    return np.where(cosd >= np.cos(np.radians(radius_deg)), area_sfc, 0.0)


def time_adjoint(res, n_lloyd, n_steps, dt, device, repeats=3):
    """Cost of the adjoint relative to the forward step on the adjoint
    configuration: dry, 2 km mountain, standard atmosphere with 1 K noise,
    a window of n_steps at dt, objective sum over a 20-degree cap at 45N/0E
    of area_sfc * p_sfc^2.  Forward: the fused FP64 step, device-resident,
    CUDA graphs.  Window forward / backward: the C-ABI calls (the backward
    recomputes every step from its checkpoint), CUDA events on the library
    stream around each call, mean over the repeats."""
    from game_archived_gb300 import abi, cases, structs
    from game_archived_gb300.ops import CAbiOps
    tab, m = build_model(res, 0, n_lloyd, pinned=False, mountain=MOUNTAIN)
    g = abi.GpuModel(m, abi.FP64, device=device)
    try:
        cases.build_initial_state(m, tab, "std_wind_tpert", CAbiOps(g.lib, m))
    finally:
        g.close()
    ms_fwd = time_resident(m, abi.FP64, n_steps, 3, dt, device)[0]
    mm = copy_model(m, pinned=False)
    g = abi.GpuModel(mm, abi.FP64, device=device)
    try:
        mm.config["totally_first_step_bool"][0] = 1
        lay = mm.layout
        out, bar, grad = (structs.HostStruct(lay, "state") for _ in range(3))
        w = cap_weights(mm)
        g.window_forward(mm.state_old, out, dt, n_steps)
        J = g.sfc_pressure_objective(out, w, bar)
        g.window_backward(bar, grad)
        tf, tb = [], []
        for _ in range(repeats):
            g.event_record(0)
            g.window_forward(mm.state_old, out, dt, n_steps)
            g.event_record(1)
            g.window_backward(bar, grad)
            g.event_record(2)
            g.synchronize()
            tf.append(g.event_elapsed_ms(0, 1))
            tb.append(g.event_elapsed_ms(1, 2))
    finally:
        g.close()
    wf, wb = statistics.mean(tf) / n_steps, statistics.mean(tb) / n_steps
    return {"config": f"RES_ID={res} ({grid_sizes(res)['nc']} cells), 26 layers, dry, 2 km mountain, "
                      f"{n_steps}-step window, dt={dt:g} s, objective: area-weighted p_sfc^2 over a 20-degree cap",
            "forward_fused_fp64_ms_per_step": ms_fwd,
            "window_forward_ms_per_step": wf,
            "window_backward_ms_per_step": wb,
            "adjoint_over_forward": wb / ms_fwd,
            "objective": J,
            "note": "backward recomputes each step from its checkpoint (both RK stage states kept) and runs the "
                    "hand-written adjoint kernels; window times include the host-in/host-out copy of one State"}


def time_large_run(res, n_lloyd, steps, dt, device, window=24):
    """The large configuration: RES_ID=7 (163842 cells, 491520 edges), 26
    layers, the 2 km Gaussian mountain, moist build with its five non-main
    constituents advected as seeded log-normal (sigma 0.5) x exp(-z / 3 km)
    fields, dt = 50 s, `steps` mixed-precision steps (1728 = 24 h),
    device-resident with CUDA graphs.  The adjoint window runs on the same
    moist model and initial state: `window` FP64 steps of dt with each step's
    start state and lagged fields checkpointed, the step recomputed with both
    RK stage states in the backward sweep.  Device memory is read
    with cudaMemGetInfo after each part, less what was in use before the
    library's first allocation."""
    from game_archived_gb300 import abi, cases, structs
    from game_archived_gb300.ops import CAbiOps
    import numpy as np
    base = device_used_bytes(device)
    tab, m = build_model(res, 1, n_lloyd, pinned=False, mountain=MOUNTAIN)
    g = abi.GpuModel(m, abi.FP64, device=device)
    try:
        cases.build_initial_state(m, tab, "tracers", CAbiOps(g.lib, m))
    finally:
        g.close()
    lay = m.layout
    mem = []
    t0 = time.perf_counter()
    ms, launches, _, _, finite = time_resident(m, abi.MIXED, steps, 3, dt, device, mem_used=mem)
    wall = time.perf_counter() - t0
    fwd = {"steps": steps, "dt_s": dt, "steps_per_s": 1000.0 / ms, "ms_per_step": ms,
           "simulated_hours": steps * dt / 3600.0, "wall_s_incl_setup": wall,
           "device_bytes_in_use": int(mem[0] - base), "gpu_launches": int(launches), "finite": finite,
           "state_struct_bytes": int(lay.sizes["state"])}
    # adjoint window of the moist step from the same initial state
    md = copy_model(m, pinned=False)
    g = abi.GpuModel(md, abi.FP64, device=device)
    try:
        md.config["totally_first_step_bool"][0] = 1
        out, bar, grad = (structs.HostStruct(lay, "state") for _ in range(3))
        w = cap_weights(md)
        g.event_record(0)
        g.window_forward(md.state_old, out, dt, window)
        g.event_record(1)
        J = g.sfc_pressure_objective(out, w, bar)
        g.event_record(2)
        g.window_backward(bar, grad)
        g.event_record(3)
        g.synchronize()
        used = device_used_bytes(device) - base
        tf, tb = g.event_elapsed_ms(0, 1), g.event_elapsed_ms(2, 3)
        ok = bool(np.isfinite(grad["rho"]).all() and np.isfinite(grad["wind"]).all())
    finally:
        g.close()
    adj = {"build": "moist (six constituents), the forward run's initial state", "window_steps": window, "dt_s": dt,
           "window_forward_ms_per_step": tf / window, "window_backward_ms_per_step": tb / window,
           "steps_per_s_backward": 1000.0 * window / tb, "device_bytes_in_use": int(used),
           "objective": J, "finite": ok}
    return {"config": f"RES_ID={res} ({grid_sizes(res)['nc']} cells, {grid_sizes(res)['ne']} edges), 26 layers, "
                      f"2 km Gaussian mountain, moist build, 5 advected constituents log-normal(0.5) x exp(-z/3 km), "
                      f"mixed precision, dt={dt:g} s",
            "forward": fwd, "adjoint": adj}


DIFF_SWITCHES = ("momentum_diff_h", "momentum_diff_v", "temperature_diff_h", "temperature_diff_v", "mass_diff_h",
                 "mass_diff_v")


def time_diffusion(model0, steps, warmup, dt, device, base_ms):
    """The headline workload with every diffusion switch on (the reference's
    ideal and operational run scripts) and a seeded TKE of 0.5-1 J/kg:
    device-resident steps/s in both precisions, the ratio to the step
    without diffusion, and the per-step time of the diffusion kernels (kd_*)
    from the profiled pass."""
    import numpy as np
    from game_archived_gb300 import abi
    m = copy_model(model0, pinned=False)
    for s in DIFF_SWITCHES:
        m.config[s][0] = 1
    m.irrev["tke"][:] = 0.5 + 0.5 * np.random.default_rng(5).random(m.irrev["tke"].size)
    out = {"config": "as the headline workload, momentum, temperature and mass diffusion on (horizontal and "
                     "vertical), TKE 0.5-1 J/kg seeded"}
    for prec, name in ((abi.MIXED, "mixed"), (abi.FP64, "fp64")):
        ms, launches, _, prof, ok = time_resident(m, prec, steps, warmup, dt, device, profile=True)
        kd = {k: v[0] / steps for k, v in prof.items() if k.startswith("kd_")}
        out[name] = {"steps_per_s": 1000.0 / ms, "ms_per_step": ms, "over_no_diffusion": ms / base_ms[name],
                     "diffusion_kernels_ms_per_step_profiled": sum(kd.values()), "kernels": kd,
                     "gpu_launches": int(launches), "finite": bool(ok)}
    return out


def time_output(model0, device, n_wind=4, repeats=10):
    """The output diagnostics of write_out (game_gpu_write_out_fields) on the
    headline workload's state, device-resident, with the lowest-layer wind of
    n_wind steps recorded on the device: the device-only pass (every field
    computed, nothing copied to the host), and the full call with every field
    on the native grid and on the lat-lon grid written to host memory.  The
    CPU side is the oracle's restatement of write_out (the reference's
    algorithm, OpenMP on all host threads) plus its interpolate_to_ll of
    every horizontal slice, on the same state."""
    import numpy as np
    from game_archived_gb300 import abi
    from oracle import bind
    m = copy_model(model0, pinned=False)
    lay = m.layout
    out = {"config": f"write_out's fields of the headline state: 11 surface, 8 model-layer, 7 pressure-level "
                     f"fields on {lay.nc} cells and on the {lay.n_latlon}-point lat-lon grid (every slice, as "
                     f"the GRIB path), 10 m wind over {n_wind} recorded steps"}
    g = abi.GpuModel(m, abi.FP64, resident=True, device=device)
    try:
        g.sync_to_device(m.state_new)
        for t in range(n_wind):
            g.record_wind_lowest(m.state_new, t)
        for _ in range(3):
            g.output_fields(m.state_new, None, n_wind, native=False, latlon=False)
        g.synchronize()
        g.kernel_launches(reset=True)
        g.event_record(0)
        for _ in range(repeats):
            g.output_fields(m.state_new, None, n_wind, native=False, latlon=False)
        g.event_record(1)
        g.synchronize()
        dev_ms = g.event_elapsed_ms(0, 1) / repeats
        launches = g.kernel_launches(reset=True) / repeats
        # per-kernel-group times (events around each launch group, a separate
        # pass: the events serialise the launches)
        g.profile(True)
        for _ in range(repeats):
            g.output_fields(m.state_new, None, n_wind, native=False, latlon=True)
        g.synchronize()
        g.profile(False)
        prof = {k: v[0] / repeats for k, v in g.profile_results().items() if k.startswith("out_")}
        bufs = g.output_fields(m.state_new, None, n_wind, native=True, latlon=True)
        g.transfer_bytes(reset=True)
        t0 = time.perf_counter()
        for _ in range(repeats):
            g.output_fields(m.state_new, None, n_wind, native=True, latlon=True, buffers=bufs)
        full_ms = (time.perf_counter() - t0) * 1000.0 / repeats
        h2d, d2h = g.transfer_bytes(reset=True)
    finally:
        g.close()
    out["gpu"] = {"device_ms": dev_ms, "call_ms_with_host_copies": full_ms, "d2h_bytes_per_call": int(d2h / repeats),
                  "h2d_bytes_per_call": int(h2d / repeats), "gpu_launches_per_call": launches,
                  "kernel_groups_ms_profiled_with_latlon": prof}
    # the oracle on the host cores: one untimed call, then timed calls
    mo = copy_model(model0, pinned=False)
    orc = bind.Oracle(mo)
    lo = lay.n_vectors - lay.vpl
    wl = np.concatenate([mo.state_new["wind"][lo:lo + lay.ne]] * n_wind)
    nc, nl = lay.nc, lay.nl

    def cpu_call():
        f = bind.write_out_fields(orc, mo.state_new, wl, n_wind)
        fields = [f[k] for k in bind.OUTPUT_SURFACE] + [mo.diagnostics["temperature"], mo.diagnostics["u_at_cell"],
                                                        mo.diagnostics["v_at_cell"]]
        fields += [f[k] for k in bind.OUTPUT_LAYERS]
        for a in fields:
            for k in range(len(a) // nc):
                bind.interpolate_to_ll(orc, a[k * nc:(k + 1) * nc])
        for k in bind.OUTPUT_PLEVELS:
            a = f[k].reshape(nc, 6)
            for j in range(6):
                bind.interpolate_to_ll(orc, np.ascontiguousarray(a[:, j]))
        for k in range(nl + 1):
            bind.interpolate_to_ll(orc, mo.state_new["wind"][k * lay.vpl:k * lay.vpl + nc])
    cpu_call()
    times = []
    for _ in range(2):
        t0 = time.perf_counter()
        cpu_call()
        times.append(time.perf_counter() - t0)
    cpu_ms = 1000.0 * min(times)
    out["cpu_oracle"] = {"call_ms": cpu_ms, "cores": os.cpu_count(), "kind": "port"}
    out["speedup_call_with_host_copies"] = cpu_ms / full_ms
    return out


def cpu_baseline(model0, dt, max_seconds=25.0):
    """oracle on all host threads; bounded number of steps"""
    from game_archived_gb300 import driver
    from oracle.bind import Oracle
    m = copy_model(model0, pinned=False)
    o = Oracle(m)
    driver.start(m, o.linear_combine_two_states)
    times = []
    t = 0.0
    t_start = time.perf_counter()
    while True:
        t0 = time.perf_counter()
        driver.step(m, o.linear_combine_two_states, o.manage_rkhevi, dt, t)
        times.append(time.perf_counter() - t0)
        t += dt
        if len(times) >= 2 and (time.perf_counter() - t_start > max_seconds or len(times) >= 8):
            break
    steady = times[1:] if len(times) > 1 else times
    return statistics.median(steady), len(times)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def allreduce_max(x, world):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def run_ours(args):
    from game_archived_gb300 import abi, workloads
    from game_archived_gb300.ops import CAbiOps
    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    name = HEADLINE
    res, moist, case, mountain, dt, _ = workloads.CONFIGS[name]
    if rank == 0:
        workloads.prepare(name, args.n_lloyd)
    barrier(world)
    tab, model0 = workloads.load(name, args.n_lloyd)
    g = abi.GpuModel(model0, abi.FP64, device=local)
    try:
        workloads.initial_state(name, tab, model0, CAbiOps(g.lib, model0))
    finally:
        g.close()
    n_const = model0.layout.n_const

    barrier(world)
    i64, i32, i32f, ie = {}, {}, {}, {}
    ms64, _, _, _, ok64 = time_resident(model0, abi.FP64, args.steps, args.warmup, dt, local,
                                        min_seconds=args.min_seconds, world=world, info=i64)
    barrier(world)
    # the mixed step with its vertical eliminations in FP64 (for comparison)
    ms32f, _, _, _, ok32f = time_resident(model0, abi.MIXED, args.steps, args.warmup, dt, local,
                                          min_seconds=args.min_seconds, world=world, double_float=0,
                                          info=i32f)
    barrier(world)
    sampler = ClockSampler(local)
    ms32, launches, clocks, prof, ok32 = time_resident(model0, abi.MIXED, args.steps, args.warmup, dt, local,
                                                       sampler=sampler, profile=True, min_seconds=args.min_seconds,
                                                       world=world, info=i32)
    barrier(world)
    ms32_max = allreduce_max(ms32, world)
    ms32f_max = allreduce_max(ms32f, world)
    ms64_max = allreduce_max(ms64, world)
    e2e_sec, h2d, d2h = time_e2e(model0, abi.MIXED, args.steps, min(args.warmup, 3), dt, local,
                                 min_seconds=args.min_seconds, world=world, info=ie)
    e2e_max = allreduce_max(e2e_sec, world)
    if rank != 0:
        barrier(world)
        return
    value = world * 1000.0 / ms32_max
    peak, peak_kind = measured_peak()
    # dominant kernel of the mixed step
    kb = kernel_bytes(res, n_const, 4)
    total_ms = sum(v[0] for v in prof.values())
    dom = max(prof.items(), key=lambda kv: kv[1][0])
    dom_name, (dom_ms, dom_n) = dom
    dom_bytes_step, dom_launch_per_step = kb.get(dom_name, (None, 1))
    avg_launch_ms = dom_ms / dom_n
    bytes_per_launch = dom_bytes_step / dom_launch_per_step if dom_bytes_step else None
    achieved = bytes_per_launch / (avg_launch_ms * 1e-3) / 1e9 if bytes_per_launch else None
    step_bytes = b_step(res, n_const, 8, 8, 4)
    kernels = {k: {"ms_per_launch": v[0] / v[1], "share": v[0] / total_ms, "launches": v[1]} for k, v in prof.items()}
    for k, v in kernels.items():
        if k in kb:
            bpl = kb[k][0] / kb[k][1]
            v["algorithmic_bytes_per_launch"] = bpl
            v["gbs"] = bpl / (v["ms_per_launch"] * 1e-3) / 1e9
    g = grid_sizes(res)
    prof_traffic, prof_src = read_profile(dom_name, "dram_bytes_per_launch")
    line = {
        "metric": METRIC,
        "value": value,
        "unit": "steps/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "timed_steps": i32["timed_steps"],
        "ms_per_step": ms32_max,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32+f64",
        "data": "synthetic",
        "config": {"workload": workload_text(name, res, g, dt),
                   "precision": "mixed: FP32 horizontal operators; FP64 state, tendencies and mass-flux "
                                "accumulation; vertical eliminations in double-float (48-bit significands on "
                                "the FP32 pipe)",
                   "parallelism": "replicas" if world > 1 else "single GPU",
                   "grid": f"{args.n_lloyd} Lloyd iterations",
                   "timing": f"{args.steps} steps repeated to cover >= {args.min_seconds:g} s per timed region",
                   "l2": "working set per step > L2 (state+tables+work >> 129 MB)"},
        "fp64": {"steps_per_s": world * 1000.0 / ms64_max, "ms_per_step": ms64_max,
                 "timed_steps": i64["timed_steps"]},
        "mixed_over_fp64": ms64_max / ms32_max,
        "mixed_fp64_eliminations": {"steps_per_s": world * 1000.0 / ms32f_max, "ms_per_step": ms32f_max,
                                    "timed_steps": i32f["timed_steps"]},
        "roofline": {"bound": "hbm", "kernel": dom_name,
                     "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": (achieved / peak) if achieved else None,
                     "traffic": prof_traffic, "traffic_source": prof_src, "peak_source": peak_kind},
        "roofline_step": {"algorithmic_bytes": step_bytes, "achieved": step_bytes / (ms32_max * 1e-3) / 1e9,
                          "peak": peak, "unit": "GB/s", "frac": step_bytes / (ms32_max * 1e-3) / 1e9 / peak},
        "kernels": kernels,
        "e2e": {"value": world / e2e_max, "unit": "steps/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "timed_steps": ie["timed_steps"]},
        "gpu_launches": int(launches),
        "clocks": clocks,
        "finite": bool(ok32 and ok64 and ok32f),
    }
    if not args.no_diffusion:
        line["diffusion"] = time_diffusion(model0, max(20, args.steps // 4), args.warmup, dt, local,
                                           {"mixed": ms32, "fp64": ms64})
    if not args.no_output:
        line["output"] = time_output(model0, local)
    if not args.no_adjoint:
        line["adjoint"] = time_adjoint(args.adjoint_res, None, 12, 200.0, local)
    if not args.no_large:
        line["large_run"] = time_large_run(7, None, args.large_steps, 50.0, local)
    if world == 1 and not args.no_cpu_baseline:
        sec, n = cpu_baseline(model0, dt)
        line["cpu_baseline"] = {"value": 1.0 / sec, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                                "sample": f"{n} RKHEVI steps of the same workload, FP64, OpenMP over "
                                          f"{os.cpu_count()} host threads, median of steps after the first"}
        line["cpu_1thread"] = one_thread_row(name, args.n_lloyd)
    print(json.dumps(line))
    barrier(world)


COLUMN_SOLVERS = {0: "auto", 1: "sweeps", 2: "pcr"}
SOLVER_KERNELS = ("k_waves_thomas", "k_tracers_solve", "k_tracers_sedheat", "k_vertical_tracers")


STUDY = ((6, 26, (0, 2)), (6, 64, (1, 2)), (6, 128, (1, 2)),
         (5, 128, (1, 2)), (4, 128, (0, 1, 2)), (4, 256, (0, 1, 2)), (3, 256, (1, 2)))


def column_study(args):
    """Column solvers against grid size and layer count (--column-study): the
    headline workload (moist jet) at the (RES_ID, layers) pairs of STUDY, each
    with registers (per-thread Thomas sweep in registers, 26 layers), sweeps
    (per-thread sweep in local memory, any other count), pcr (warp-
    cooperative parallel cyclic reduction) and, where it is a mix of the two,
    auto (the library's default choice); dt = --dt up to 128 layers and
    shortened in proportion above.  One JSON line per (grid, layers, solver,
    precision): device-resident steps/s and the per-step time of the
    vertical-solver kernels from the profiled pass."""
    from game_archived_gb300 import abi, cases
    from game_archived_gb300.ops import CAbiOps
    _, _, local = dist_env()
    for res, nl, solvers in STUDY:
        dt = args.dt * min(1.0, 128.0 / nl)
        tab, m = build_model(res, 1, args.n_lloyd, pinned=False, n_layers=nl)
        g = abi.GpuModel(m, abi.FP64, device=local)
        try:
            cases.build_initial_state(m, tab, "jet_moist", CAbiOps(g.lib, m))
        finally:
            g.close()
        for solver in solvers:
            for prec, name in ((abi.MIXED, "mixed"), (abi.FP64, "fp64")):
                ms, launches, _, prof, ok = time_resident(m, prec, args.steps, args.warmup, dt, local,
                                                          profile=True, column_solver=solver)
                total = sum(v[0] for v in prof.values())
                solve = {k: prof[k][0] / args.steps for k in SOLVER_KERNELS if k in prof}
                print(json.dumps({
                    "study": "column solvers", "res": res, "columns": grid_sizes(res)["nc"], "layers": nl,
                    "solver": "registers" if (solver == 0 and nl == L) else COLUMN_SOLVERS[solver],
                    "precision": name, "dt": dt,
                    "steps_per_s": 1000.0 / ms, "ms_per_step": ms, "steps": args.steps,
                    "vertical_solver_ms_per_step_profiled": solve,
                    "vertical_solver_share": sum(solve.values()) * args.steps / total,
                    "gpu_launches": int(launches), "finite": bool(ok)}), flush=True)


HEADLINE = "config3"


def _cpu_steps(name, n_lloyd, warmup, steps):
    """(median, mean) seconds per step of the oracle on the configuration's
    prepared inputs, after warmup steps; OpenMP threads as the environment
    sets them.  Loads only the oracle's library."""
    from game_archived_gb300 import driver, workloads
    from oracle.bind import Oracle
    dt = workloads.CONFIGS[name][4]
    tab, m = workloads.load(name, n_lloyd)
    o = Oracle(m)
    workloads.initial_state(name, tab, m, o)
    driver.start(m, o.linear_combine_two_states)
    t = 0.0
    for _ in range(warmup):
        driver.step(m, o.linear_combine_two_states, o.manage_rkhevi, dt, t)
        t += dt
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        driver.step(m, o.linear_combine_two_states, o.manage_rkhevi, dt, t)
        times.append(time.perf_counter() - t0)
        t += dt
    return statistics.median(times), sum(times) / len(times), times


def cpu_one_thread(args):
    """--cpu-one-thread: the oracle on one OpenMP thread (run as a child
    process with OMP_NUM_THREADS=1); prints one JSON line"""
    med, mean, _ = _cpu_steps(args.config, args.n_lloyd, 1, args.steps)
    print(json.dumps({"threads": 1, "steps": args.steps, "median_s": med, "mean_s": mean}))


def one_thread_row(name, n_lloyd, steps=2):
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--cpu-one-thread", "--config", name,
                        "--steps", str(steps), "--n-lloyd", str(n_lloyd)], env=env, capture_output=True, text=True,
                       timeout=900)
    if r.returncode != 0:
        return {"error": (r.stderr or r.stdout)[-300:]}
    d = json.loads(r.stdout.strip().splitlines()[-1])
    return {"value": 1.0 / d["median_s"], "unit": "steps/s", "cores": 1,
            "sample": f"{steps} steps after 1 warm-up step, one OpenMP thread, median"}


def run_reference(args):
    """The CPU implementation of the same workload: the oracle (the reference's
    algorithm restated in C with the reference's OpenMP loops, bit-identical to
    the reference's own build where that compiles) on all host threads, on the
    prepared inputs.  This process loads no library of the package: the grid
    and layout come from the files build() prepared (numpy), the initial
    state from the oracle's own operators."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from game_archived_gb300 import workloads
    name = args.config
    res, moist, case, mountain, dt, _ = workloads.CONFIGS[name]
    if not workloads.available(name, args.n_lloyd):
        print(json.dumps({"impl": "reference", "unavailable": "the benchmark inputs are not prepared: run "
                                                              "__graft_entry__.build() first"}))
        return
    med, mean, times = _cpu_steps(name, args.n_lloyd, args.warmup, args.steps)
    value = 1.0 / mean
    g = grid_sizes(res)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "steps/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": workload_text(name, res, g, dt), "precision": "FP64 (the reference's arithmetic)",
                   "parallelism": "OpenMP over all host threads"},
        "cpu_baseline": {"value": value, "unit": "steps/s", "cores": os.cpu_count(), "kind": "port",
                         "sample": f"{args.steps} steps after {args.warmup} warm-up steps (mean; median "
                                   f"{1.0 / med:.4g} steps/s), OpenMP over {os.cpu_count()} host threads; the "
                                   "oracle port, bit-identical to the reference's own build where that compiles "
                                   "(the reference's sources do not travel to this host)"},
        "cpu_1thread": one_thread_row(name, args.n_lloyd),
        "e2e": {"value": value, "unit": "steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def all_configs(args):
    """--all-configs: one JSON line per benchmark configuration (config1 ..
    config5): device-resident steps/s of the FP64 and the mixed step, the
    CPU oracle on all host threads and on one thread (bounded samples), on
    the configuration's own grid, state and time step"""
    from game_archived_gb300 import abi, workloads
    from game_archived_gb300.ops import CAbiOps
    _, _, local = dist_env()
    for name in args.configs.split(","):
        res, moist, case, mountain, dt, steps = workloads.CONFIGS[name]
        workloads.prepare(name)
        tab, m = workloads.load(name)
        g = abi.GpuModel(m, abi.FP64, device=local)
        try:
            workloads.initial_state(name, tab, m, CAbiOps(g.lib, m))
        finally:
            g.close()
        k = min(steps, args.steps)
        line = {"config": name, "workload": workload_text(name, res, grid_sizes(res), dt), "steps_per_block": k}
        mem = []
        for prec, key in ((abi.FP64, "gpu_fp64"), (abi.MIXED, "gpu_mixed")):
            info = {}
            ms, _, _, _, ok = time_resident(m, prec, k, args.warmup, dt, local, min_seconds=args.min_seconds,
                                            info=info, mem_used=mem)
            line[key] = {"steps_per_s": 1000.0 / ms, "ms_per_step": ms, "timed_steps": info["timed_steps"],
                         "finite": ok}
        line["mixed_over_fp64"] = line["gpu_fp64"]["ms_per_step"] / line["gpu_mixed"]["ms_per_step"]
        line["device_bytes_in_use"] = max(mem) if mem else None
        peak, _ = measured_peak()
        b = b_step(res, m.layout.n_const, 8, 8, 4)
        line["roofline_step_mixed"] = {"algorithmic_bytes": b, "frac": b / (line["gpu_mixed"]["ms_per_step"] * 1e-3)
                                       / 1e9 / peak}
        if not args.no_cpu_baseline:
            n_cpu = {4: 6, 5: 4, 6: 3, 7: 2}.get(res, 2)
            med, mean, _ = _cpu_steps(name, None, 1, n_cpu)
            line["cpu_all_threads"] = {"steps_per_s": 1.0 / med, "threads": os.cpu_count(),
                                       "sample": f"{n_cpu} steps after 1, median"}
            line["cpu_1thread"] = one_thread_row(name, workloads.n_lloyd_default(res), steps=1 if res >= 6 else 2)
        print(json.dumps(line), flush=True)


def profile_run(args):
    """--profile-run: only the device-resident mixed step of --config, --warmup
    + --steps steps (no repetition to a minimum time, no other arm), for
    profiler captures whose launch order must be the step's alone; prints one
    JSON line (not a benchmark figure)"""
    from game_archived_gb300 import abi, workloads
    from game_archived_gb300.ops import CAbiOps
    _, _, local = dist_env()
    name = args.config
    res, moist, case, mountain, dt, _ = workloads.CONFIGS[name]
    workloads.prepare(name, args.n_lloyd)
    tab, m = workloads.load(name, args.n_lloyd)
    g = abi.GpuModel(m, abi.FP64, device=local)
    try:
        workloads.initial_state(name, tab, m, CAbiOps(g.lib, m))
    finally:
        g.close()
    prec = abi.FP64 if args.precision == "fp64" else abi.MIXED
    ms, launches, _, _, ok = time_resident(m, prec, args.steps, args.warmup, dt, local, min_seconds=0.0)
    print(json.dumps({"profile_run": name, "precision": args.precision, "steps": args.steps, "warmup": args.warmup,
                      "ms_per_step": ms, "launches": launches, "finite": ok}))


def workload_text(name, res, g, dt):
    from game_archived_gb300 import workloads
    _, moist, case, mountain, _, steps = workloads.CONFIGS[name]
    what = {"baroclinic_moist": "moist (6 constituents), baroclinic jet of Jablonowski-Williamson (2006) in "
                                "thermal-wind balance + N(0, 0.5 m/s) wind noise, RH 0.7 below 8 km",
            "std_wind": "dry, ICAO standard atmosphere, u = 20 cos(lat) + N(0, 1 m/s)",
            "std_wind_tpert": "dry, ICAO standard atmosphere + N(0, 1 K), u = 20 cos(lat) + N(0, 1 m/s)",
            "tracers": "moist build, five constituents seeded log-normal x exp(-z / 3 km)"}[case]
    return (f"RKHEVI step, {name}: RES_ID={res} ({g['nc']} cells, {g['ne']} edges), 26 layers, "
            f"{'2 km Gaussian mountain' if mountain else 'flat'}, {what}, dt={dt:g} s")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=400)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--res", type=int, default=6)
    ap.add_argument("--dt", type=float, default=100.0)
    ap.add_argument("--n-lloyd", type=int, default=2000)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--no-diffusion", action="store_true")
    ap.add_argument("--no-output", action="store_true")
    ap.add_argument("--adjoint-res", type=int, default=5)
    ap.add_argument("--no-large", action="store_true", help="skip the RES_ID=7 run with five constituents")
    ap.add_argument("--large-steps", type=int, default=1728)
    ap.add_argument("--min-seconds", type=float, default=2.0,
                    help="repeat the timed steps until each timed region covers this many seconds")
    ap.add_argument("--column-study", action="store_true",
                    help="time the column solvers at 26, 64 and 128 layers instead of the headline line")
    ap.add_argument("--cpu-one-thread", action="store_true", help=argparse.SUPPRESS)
    ap.add_argument("--all-configs", action="store_true",
                    help="one line per benchmark configuration instead of the headline line")
    ap.add_argument("--configs", default="config1,config2,config3,config4,config5")
    ap.add_argument("--ncu-json", nargs="+", help="summarise ncu raw-page CSVs into --out (see ncu_json)")
    ap.add_argument("--ncu-metric-list", action="store_true",
                    help="print the metrics the summary keeps, comma-separated (for ncu --metrics)")
    ap.add_argument("--out")
    ap.add_argument("--command", default="", help="the capture command, recorded in the summary")
    ap.add_argument("--captured", default="", help="what was captured (workload, commit state), recorded")
    ap.add_argument("--config", default=HEADLINE)
    ap.add_argument("--profile-run", action="store_true",
                    help="only the resident step of --config (--precision), for profiler captures")
    ap.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    args = ap.parse_args()
    if args.cpu_one_thread:
        cpu_one_thread(args)
        return
    if args.ncu_json:
        ncu_json(args)
        return
    if args.ncu_metric_list:
        print(",".join(NCU_METRICS))
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.profile_run:
        profile_run(args)
    elif args.all_configs:
        all_configs(args)
    elif args.column_study:
        column_study(args)
    elif args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
