#!/usr/bin/env python
"""Benchmark of the FDTD step loop on GB300.

One bench step = one FDTD time step (H and E half-steps with CPML, TF/SF
plane wave and probe recording) over the whole grid of the workload.
Default workload: the 512x512x448 layered-earth configuration (c3: 16-cell
CPML, 6 conductive layers below air, vertically incident TF/SF plane wave,
256-cell surface probe line), synthetic seeded inputs; the state (~3.4 GB)
exceeds the 129 MB L2, so no L2 flush is needed between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c1|c2|c3]
  python bench.py --impl reference ...   # the CPU arm (oracle, all cores)

Prints ONE JSON line on rank 0.  Multi-GPU: one process per GPU (torchrun),
each advancing its own replica of the workload (the path has no exchange);
value = all ranks' cell-steps / max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic bytes per cell.  The reference's layout (per-cell coefficient
# arrays): H half-step read 3 H + 3 E, write 3 H = 36 B; E half-step read
# 3 E + 3 H + 6 coefficients, write 3 E = 60 B; 96 B per step.
REF_BYTES_H, REF_BYTES_E = 36, 60
# Compulsory bytes of this design: the E coefficients are a 2-byte material
# id per cell (a table of the distinct tuples in shared memory) when the grid
# has at most 32768 distinct tuples, else the six arrays; H as above.  The
# fused step (H and E in one pass, fields read from one buffer and written
# to a second): read 3 E + 3 H + the id, write 3 E + 3 H.
ID_BYTES_E = 38
FUSED_BYTES = 50
FALLBACK_HBM_GBS = 6800.0


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------- ranks

class Ranks:
    def __init__(self, join: bool = True):
        self.rank = int(os.environ.get("RANK", "0"))
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1 and join:
            import torch.distributed as dist

            os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
            dist.init_process_group("gloo", rank=self.rank, world_size=self.world)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, v: float) -> float:
        if not self.pg:
            return v
        import torch

        t = torch.tensor([v], dtype=torch.float64)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


# ----------------------------------------------------------------- clocks

class ClockSampler:
    """nvidia-smi clock / throttle samples taken during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def start(self):
        import tempfile

        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-i", str(self.gpu), "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self) -> dict:
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.path)
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def measured_hbm_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return FALLBACK_HBM_GBS, "fallback"


def ncu_traffic(workload: str) -> dict:
    """DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum)
    of this workload's kernels from the committed ncu summary
    (profiles/ncu_traffic.json)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.json")
    try:
        with open(path) as f:
            return json.load(f).get(workload, {})
    except (OSError, ValueError):
        return {}


# ----------------------------------------------------------------- CPU arm

def cpu_oracle_rate(w, target_s: float, max_steps: int, warmup: int = 3):
    """Times the FP32 oracle (OpenMP, all host threads) on the workload's grid
    for a bounded number of steps after `warmup` untimed ones; returns
    (Mcell-steps/s, steps, seconds, OpenMP threads used)."""
    import oracle
    from maxwell_solver_gb300.workloads import materials, probe_locations, sources

    oracle.build()
    oracle.set_threads(os.cpu_count() or 1)  # torchrun sets OMP_NUM_THREADS=1
    T = max_steps + warmup + 1
    o = oracle.OracleSim("f32")
    o.set_params(pml=w.pml, tfsf_width=w.pml + 5)
    I, J, K = w.dims
    o.set_const(np.float32([w.fctr, w.delX, w.delT]), np.int32([T, I, J, K, w.n_probes]))
    pw, cur = sources(w, T)
    o.set_source(cur)
    if w.n_probes:
        o.set_antenna_locations(np.asfortranarray(probe_locations(w)))
    for flag, arr in materials(w).items():
        o.update_material(flag, arr)
    o.ready_simulation()
    if w.mode == 5:
        o.set_incidence(*w.angles)
    o.init_1d(1.0, pw)
    for n in range(warmup):
        o.step(n, w.mode)
    n, t0 = warmup, time.perf_counter()
    while n < warmup + max_steps:
        o.step(n, w.mode)
        n += 1
        if time.perf_counter() - t0 >= target_s:
            break
    dt = time.perf_counter() - t0
    steps = n - warmup
    o.close()
    return w.cells * steps / dt / 1e6, steps, dt, oracle.threads()


def run_reference(args, ranks):
    from maxwell_solver_gb300.workloads import WORKLOADS

    if ranks.rank != 0:
        return None
    w = WORKLOADS[args.workload]
    steps = max(1, min(args.steps, 200))
    warmup = max(3, args.warmup)
    rate, done, secs, cores = cpu_oracle_rate(w, target_s=10.0, max_steps=steps, warmup=warmup)
    sample = (f"{w.dims[0]}x{w.dims[1]}x{w.dims[2]} grid of workload {w.name}, {done} FDTD "
              f"steps ({secs:.1f} s) of the FP32 CPU restatement, OpenMP {cores} threads")
    return {
        "impl": "reference", "metric": "Mcell-steps/s", "value": round(rate, 3),
        "unit": "Mcell-steps/s", "n_gpus": args.gpus, "steps": done, "warmup": warmup,
        "ms_per_step": round(secs / done * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {**workload_config(w), "parallelism": f"replicas x{args.gpus}"},
        "cpu_baseline": {"value": round(rate, 3), "unit": "Mcell-steps/s", "cores": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": round(rate, 3), "unit": "Mcell-steps/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
        "note": ("the reference ships no CPU implementation of the step loop; its GPU "
                 "kernels run only under MATLAB's MEX runtime, so the reference arm is the "
                 "oracle's restatement of them, pinned bit-exact to the reference's sources"),
    }


def workload_config(w):
    return {"workload": f"{w.name}: {w.dims[0]}x{w.dims[1]}x{w.dims[2]} Yee grid",
            "cells": w.cells, "pml": w.pml, "media": w.media, "tfsf_mode": w.mode,
            "probes": w.n_probes, "config_steps": w.steps,
            **({"incidence_rad": [round(a, 6) for a in w.angles]} if w.mode == 5 else {}),
            "l2": (f"inputs larger than L2 (fields+coefficients {w.cells * 48 / 1e6:.0f} MB"
                   " > 129 MB), no flush needed" if w.cells * 48 > 129e6 else
                   f"state {w.cells * 48 / 1e6:.0f} MB fits in L2: not a headline configuration")}


# ----------------------------------------------------------------- GPU arm

def run_ours(args, ranks):
    import ctypes
    import tempfile

    from maxwell_solver_gb300 import _native, info, launch_count, simFDTD
    from maxwell_solver_gb300.simfdtd import _check
    from maxwell_solver_gb300.workloads import WORKLOADS, materials, probe_locations, setup, sources

    # a fresh autotune cache (unless --tune-cache names one): the end-to-end
    # leg, which runs first, pays the autotuner's trial steps as a first
    # drop-in call on this machine would
    if args.tune_cache:
        os.environ["FDTD_TUNE_CACHE"] = args.tune_cache
    else:
        tune_dir = tempfile.mkdtemp(prefix="fdtd_tune_")
        os.environ["FDTD_TUNE_CACHE"] = os.path.join(tune_dir, "autotune.txt")
    lib = _native.load()
    _check(lib.fdtd_set_device(ranks.local))
    w = WORKLOADS[args.workload]
    W, K = args.warmup, args.steps
    cells = w.cells

    # end to end through the public per-op interface (host buffers, H2D of
    # materials and sources, D2H of probes and a field, all inside the timing)
    # (every rank runs its replica's; the whole job's rate is the cell-steps
    # of all ranks over the slowest rank's time)
    e2e = None
    if not args.no_e2e:
        e2e_steps = args.e2e_steps or w.steps
        ranks.barrier()
        e2e = run_e2e(w, e2e_steps, simFDTD, materials, probe_locations, sources)
        slowest = ranks.max(e2e["seconds"])
        e2e["value"] = round(cells * e2e_steps * ranks.world / slowest / 1e6, 2)
        e2e["seconds"] = round(slowest, 3)

    KP = max(8, min(64, K // 4)) // 2 * 2  # per-kernel profiled steps (even: fused pairs)
    T = W + K + KP
    P = setup(simFDTD, w, steps=T)
    h = int(P[0])
    inf = info(P)
    simFDTD("Synchronize", P)

    simFDTD("StepN", P, np.int32([0, W, w.mode]))
    simFDTD("Synchronize", P)
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    gpu_index = int(vis) if vis.isdigit() else ranks.local
    clocks = ClockSampler(gpu_index)
    ranks.barrier()
    clocks.start()
    n0 = launch_count()
    _check(lib.fdtd_event_record(h, 0))
    simFDTD("StepN", P, np.int32([W, K, w.mode]))
    _check(lib.fdtd_event_record(h, 1))
    simFDTD("Synchronize", P)
    ms = ctypes_float()
    _check(lib.fdtd_event_elapsed_ms(h, 0, 1, ms))
    launches = launch_count() - n0
    clk = clocks.stop()
    ranks.barrier()
    ms_max = ranks.max(ms.value)

    # per-kernel device time, measured live with CUDA events around every
    # launch (on the handle's stream, where the kernels run)
    acc = (ctypes.c_float * 6)()
    _check(lib.fdtd_profile_steps(h, W + K, KP, w.mode, None, ctypes.byref(acc)))
    t_h, t_e, t_o, t_hc, t_ec, t_f = (acc[i] / KP for i in range(6))
    simFDTD("DeleteSimulation", P)

    peak, peak_kind = measured_hbm_peak()
    value = cells * K * ranks.world / (ms_max / 1e3) / 1e6
    step_ms = ms.value / K
    e_bytes = ID_BYTES_E if inf["coef_mode"] == 1 else REF_BYTES_E
    gbs = lambda b, t_ms: b * cells / (t_ms / 1e3) / 1e9 if t_ms > 0 else 0.0  # noqa: E731
    tr = ncu_traffic(w.name)
    tr_e, tr_h = tr.get("k_half_e_bytes_per_launch"), tr.get("k_half_h_bytes_per_launch")
    kern = {
        "E": {"kernel": "k_half_e_tma (E curl + CPML Y, Z)", "alg_bytes_per_cell": e_bytes,
              "avg_launch_ms": round(t_ec, 5), "achieved": round(gbs(e_bytes, t_ec), 1),
              "frac": round(gbs(e_bytes, t_ec) / peak, 4), "traffic": tr_e,
              "half_step_ms": round(t_e, 5)},
        "H": {"kernel": "k_half_h_tma (H curl + CPML X, Y, Z)", "alg_bytes_per_cell": REF_BYTES_H,
              "avg_launch_ms": round(t_hc, 5), "achieved": round(gbs(REF_BYTES_H, t_hc), 1),
              "frac": round(gbs(REF_BYTES_H, t_hc) / peak, 4), "traffic": tr_h,
              "half_step_ms": round(t_h, 5)},
    }
    fused = t_f > 0
    if fused:  # the steps ran as the fused pass (the half-step kernels did not run)
        f_bytes = FUSED_BYTES if inf["coef_mode"] == 1 else FUSED_BYTES + 22
        kern = {"F": {"kernel": "k_step_fused (H and E curl + CPML Y, Z and H X, one pass)",
                      "alg_bytes_per_cell": f_bytes, "avg_launch_ms": round(t_f, 5),
                      "achieved": round(gbs(f_bytes, t_f), 1),
                      "frac": round(gbs(f_bytes, t_f) / peak, 4),
                      "traffic": tr.get("k_step_fused_bytes_per_launch"),
                      "passes_ms": round(t_e, 5)}}
        dom = "F"
    else:
        dom = "E" if t_ec >= t_hc else "H"
    d = kern[dom]
    step_comp = (kern["F"]["alg_bytes_per_cell"] if fused else e_bytes + REF_BYTES_H)
    step_bytes = tr.get("step_dram_bytes_fused" if fused else "step_dram_bytes")
    roofline = {
        "bound": "hbm", "kernel": d["kernel"], "achieved": d["achieved"], "peak": peak,
        "unit": "GB/s", "frac": d["frac"], "traffic": d["traffic"],
        "peak_source": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs, copy bandwidth)",
        "alg_bytes_per_cell": d["alg_bytes_per_cell"], "units_per_launch": cells,
        "avg_launch_ms": d["avg_launch_ms"],
        "convention": "compulsory bytes of this design (fused step: read 3 E + 3 H + a "
                      "2-byte material id, write 3 E + 3 H; half-step kernels: E read 3 E + "
                      "3 H + the id, write 3 E, H read 3 H + 3 E, write 3 H) / the kernel's "
                      "average launch time, CUDA events on the handle's stream",
        "kernels": kern,
        "step": {"ms": round(step_ms, 5),
                 "compulsory_bytes_per_cell": step_comp,
                 "achieved": round(gbs(step_comp, step_ms), 1),
                 "frac": round(gbs(step_comp, step_ms) / peak, 4),
                 "dram_bytes_per_step": step_bytes,
                 "dram_frac": (round(step_bytes / (step_ms / 1e3) / 1e9 / peak, 4)
                               if step_bytes else None),
                 "probe_gather_ms": round(t_o, 5)},
        "reference_layout": {
            "bytes_per_cell_step": REF_BYTES_H + REF_BYTES_E,
            "note": "the reference's per-cell coefficient layout (H 36 B, E 60 B); the "
                    "material ids read 2 B for its 24 B of coefficients, so this can "
                    "exceed 1",
            "step_frac": round(gbs(REF_BYTES_H + REF_BYTES_E, step_ms) / peak, 4),
            **({"E_frac": round(gbs(REF_BYTES_E, t_ec) / peak, 4),
                "H_frac": round(gbs(REF_BYTES_H, t_hc) / peak, 4)} if not fused else
               {"fused_frac": round(gbs(REF_BYTES_H + REF_BYTES_E, t_f) / peak, 4)})},
        "traffic_source": tr.get("source"),
    }

    # the batched, served, per-cell coefficient and CPU legs: one GPU only (N = 1)
    solo = ranks.world == 1
    coef_arrays = None
    if solo and not args.no_coef_arrays:
        coef_arrays = run_coef_arrays("c2", 200, 5)
    cpu = None
    if solo and not args.no_cpu:
        rate, done, secs, cores = cpu_oracle_rate(w, target_s=args.cpu_seconds, max_steps=2000)
        cpu = {"value": round(rate, 3), "unit": "Mcell-steps/s", "cores": cores,
               "kind": "port",
               "sample": f"{w.dims[0]}x{w.dims[1]}x{w.dims[2]} grid, {done} steps "
                         f"({secs:.1f} s) of the FP32 oracle, OpenMP {cores} threads"}

    served = None
    if solo and not args.no_serve:
        served = run_served(args.serve_requests,
                            [float(x) for x in args.serve_loads.split(",") if x],
                            policy=args.serve_policy)

    batched = None
    if solo and not args.no_batch:
        batched = run_batched(args.batch_grids)
    ranks.close()
    if ranks.rank != 0:
        return None
    return {
        "metric": "Mcell-steps/s", "value": round(value, 2), "unit": "Mcell-steps/s",
        "n_gpus": ranks.world, "steps": K, "warmup": W, "ms_per_step": round(ms_max / K, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded spheres/layers, Gaussian-modulated plane wave)",
        "config": {**workload_config(w), "parallelism": f"replicas x{ranks.world}"},
        "timed": ("fdtd_step_n: pairs of steps as the fused H+E pass with its x-slab, face "
                  "and fix-up passes and the probe gather" if inf["fused"] else
                  "fdtd_step_n: H and E curl kernels, their face passes, the E x-slab pass "
                  "and the probe gather") + ", replayed as CUDA graphs",
        "tuned": {"fused": inf["fused"], "zchunk_f": inf["zchunk_f"],
                  "tile_h": ("64x8", "32x16", "128x4")[inf["tile_h"]],
                  "tile_e": ("64x8", "32x16", "128x4")[inf["tile_e"]],
                  "zchunk_h": inf["zchunk_h"], "zchunk_e": inf["zchunk_e"],
                  "coef_mode": inf["coef_mode"], "num_materials": inf["num_materials"]},
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": e2e,
        "clocks": clk,
        "gpu_launches": int(launches),
        "coef_arrays": coef_arrays,
        "served": served,
        "batched": batched,
    }


def ctypes_float():
    import ctypes

    return ctypes.c_float(0.0)


def run_coef_arrays(name: str, steps: int, warmup: int):
    """The reference's coefficient layout: six per-cell E coefficient arrays
    (FDTD_COEF=arrays; 60 B per cell in the E half-step) instead of 2-byte
    material ids, on the named workload: Mcell-steps/s and the E kernel's
    roofline in those bytes."""
    import ctypes

    from maxwell_solver_gb300 import _native, info, simFDTD
    from maxwell_solver_gb300.simfdtd import _check
    from maxwell_solver_gb300.workloads import WORKLOADS, setup

    lib = _native.load()
    w = WORKLOADS[name]
    KP = 16
    os.environ["FDTD_COEF"] = "arrays"
    try:
        P = setup(simFDTD, w, steps=warmup + steps + KP)
    finally:
        del os.environ["FDTD_COEF"]
    h = int(P[0])
    inf = info(P)
    simFDTD("StepN", P, np.int32([0, warmup, w.mode]))
    _check(lib.fdtd_event_record(h, 0))
    simFDTD("StepN", P, np.int32([warmup, steps, w.mode]))
    _check(lib.fdtd_event_record(h, 1))
    simFDTD("Synchronize", P)
    ms = ctypes_float()
    _check(lib.fdtd_event_elapsed_ms(h, 0, 1, ms))
    acc = (ctypes.c_float * 6)()
    _check(lib.fdtd_profile_steps(h, warmup + steps, KP, w.mode, None, ctypes.byref(acc)))
    simFDTD("DeleteSimulation", P)
    peak, _ = measured_hbm_peak()
    t_ec = acc[4] / KP
    ach = REF_BYTES_E * w.cells / (t_ec / 1e3) / 1e9 if t_ec > 0 else 0.0
    return {"workload": f"{w.name}: {w.dims[0]}x{w.dims[1]}x{w.dims[2]}, per-cell coefficient "
                        "arrays (FDTD_COEF=arrays)",
            "coef_mode": inf["coef_mode"], "steps": steps,
            "value": round(w.cells * steps / (ms.value / 1e3) / 1e6, 2), "unit": "Mcell-steps/s",
            "ms_per_step": round(ms.value / steps, 5),
            "E_kernel": {"alg_bytes_per_cell": REF_BYTES_E, "avg_launch_ms": round(t_ec, 5),
                         "achieved": round(ach, 1), "frac": round(ach / peak, 4)}}


def run_e2e(w, K, simFDTD, materials, probe_locations, sources):
    """A whole solve through the per-op simFDTD calls: create, set-up (with
    the autotuner's trial steps when the shape is not in its cache), upload
    of the media and sources, K steps, readout of the probes and Ez."""
    I, J, K3 = w.dims
    T = K
    mats = materials(w)
    pw, cur = sources(w, T)
    loc = np.asfortranarray(probe_locations(w))
    ijk = w.cells
    t0 = time.perf_counter()
    P = simFDTD("CreateSimulation")
    simFDTD("SetParams", P, np.float64([w.pml, w.pml + 5, 3, 1, 0.08, 1, 0.8, 0]))
    simFDTD("SetConst", P, np.float32([w.fctr, w.delX, w.delT]), np.int32([T, I, J, K3, w.n_probes]))
    simFDTD("SetSource", P, cur)
    simFDTD("SetAntennaLocations", P, loc)
    for flag, arr in mats.items():
        simFDTD("UpdateMaterial", P, np.int32(flag), arr)
    simFDTD("ReadySimulation", P)
    if w.mode == 5:
        simFDTD("SetIncidence", P, np.float64(w.angles))
    simFDTD("Init1D", P, np.float32(1.0), pw)
    simFDTD("UpdateCuda", P)
    simFDTD("ResetFieldAll", P)
    m = w.mode
    for n in range(K):
        tm = np.array([n, m], dtype=np.int32)
        simFDTD("UpdateH_All", P)
        simFDTD("UpdateH_PlaneWave", P, tm)
        simFDTD("UpdateH_PML", P)
        simFDTD("UpdateE_All", P)
        simFDTD("UpdateE_PlaneWave", P, tm)
        simFDTD("UpdateE_PML", P)
    probes = simFDTD("OutputProbes", P, np.uint32(T * w.n_probes * 6))
    ez = simFDTD("OutputVis", P, np.uint32(ijk), np.int32(3))
    simFDTD("DeleteSimulation", P)
    dt = time.perf_counter() - t0
    assert np.isfinite(ez).all() and np.isfinite(probes).all()
    # host -> device: the six material arrays (UpdateMaterial copies each once;
    # UpdateCuda recomputes from the device copies), the two waveforms, the
    # probe locations
    h2d = 6 * ijk * 4 + 2 * T * 4 + loc.size * 4
    d2h = ijk * 4 + probes.size * 4
    return {"value": round(ijk * K / dt / 1e6, 2), "unit": "Mcell-steps/s",
            "h2d_bytes_per_step": int(round(h2d / K)), "d2h_bytes_per_step": int(round(d2h / K)),
            "seconds": round(dt, 6), "steps": K,
            "path": "simFDTD per-op calls (6 per step, as highfrequency.m) for the "
                    "configuration's step count, incl. set-up with the autotuner's trial "
                    "steps (empty tune cache), material/source upload, probe + Ez readout"}


def run_batched(n_grids: int, batched_only: bool = False):
    """Batched configuration c4: the same heterogeneous solves run one at a
    time through the plain solver (fdtd_step_n per grid) and together in one
    batch (one H + one E launch per step for all of them); solves/s of both,
    on the same handles (reset in between), and a bitwise identity check of
    members between the two runs."""
    from maxwell_solver_gb300 import simFDTD
    from maxwell_solver_gb300.batch import Batch
    from maxwell_solver_gb300.workloads import batch_mix, setup_grid

    mix = batch_mix(n_grids)
    t0 = time.perf_counter()
    handles = [setup_grid(simFDTD, s) for s in mix]
    for P in handles:
        simFDTD("Synchronize", P)
    t_setup = time.perf_counter() - t0
    check = list(range(0, len(mix), max(1, len(mix) // 8)))

    t_one = t_ops = None
    ref = {}
    if not batched_only:
        # one at a time through fdtd_step_n (graph-replayed fused steps)
        t0 = time.perf_counter()
        for P, s in zip(handles, mix):
            simFDTD("StepN", P, np.int32([0, s.steps, s.mode]))
            simFDTD("Synchronize", P)
        t_one = time.perf_counter() - t0
        ref = {g: simFDTD("OutputVis", handles[g], np.uint32(mix[g].cells), np.int32(3))
               for g in check}
        # one at a time through the per-op calls (6 per step, as highfrequency.m)
        for P in handles:
            simFDTD("ResetFieldAll", P)
        t0 = time.perf_counter()
        for P, s in zip(handles, mix):
            for n in range(s.steps):
                tm = np.array([n, s.mode], dtype=np.int32)
                simFDTD("UpdateH_All", P)
                simFDTD("UpdateH_PlaneWave", P, tm)
                simFDTD("UpdateH_PML", P)
                simFDTD("UpdateE_All", P)
                simFDTD("UpdateE_PlaneWave", P, tm)
                simFDTD("UpdateE_PML", P)
            simFDTD("Synchronize", P)
        t_ops = time.perf_counter() - t0

    for P in handles:
        simFDTD("ResetFieldAll", P)
        simFDTD("Synchronize", P)
    b = Batch()
    t0 = time.perf_counter()
    for P, s in zip(handles, mix):
        b.add(P, 0, s.steps, s.mode)
    b.run()
    t_batch = time.perf_counter() - t0
    zrun = b.zrun
    b.close()
    same = all(np.array_equal(ref[g], simFDTD("OutputVis", handles[g], np.uint32(mix[g].cells),
                                              np.int32(3))) for g in ref)
    for P in handles:
        simFDTD("DeleteSimulation", P)
    cell_steps = sum(s.cells * s.steps for s in mix)
    rate = lambda t: None if t is None else round(len(mix) / t, 3)  # noqa: E731
    return {
        "workload": f"c4: {len(mix)} grids, axes U{{32..128}}, 8-cell CPML, 0-10 spheres, "
                    "TF/SF oblique plane wave (mode 5, seeded angles), f0 U[10,60] GHz, "
                    "steps U[300,1500] (seed 3)",
        "solves": len(mix),
        "batched_solves_per_s": rate(t_batch),
        "one_at_a_time_solves_per_s": rate(t_one),
        "one_at_a_time_per_op_solves_per_s": rate(t_ops),
        "speedup": None if t_one is None else round(t_one / t_batch, 2),
        "speedup_vs_per_op": None if t_ops is None else round(t_ops / t_batch, 2),
        "batched_Mcell_steps_per_s": round(cell_steps / t_batch / 1e6, 1),
        "seconds": {"batched": round(t_batch, 3),
                    "one_at_a_time": None if t_one is None else round(t_one, 3),
                    "one_at_a_time_per_op": None if t_ops is None else round(t_ops, 3),
                    "setup": round(t_setup, 2)},
        "zrun": zrun,
        "identical_results": bool(same), "members_compared": len(ref),
        "timing": "wall clock, fields resident, setup excluded; one at a time = fdtd_step_n "
                  "per grid (graph-replayed fused steps) and, separately, the per-op calls",
    }


def _pct(v, p):
    """Nearest-rank percentile (the server's own statistic)."""
    v = sorted(v)
    k = min(len(v), max(1, math.ceil(p / 100.0 * len(v) - 1e-9)))
    return v[k - 1]


def _lat_summary(lat, makespan):
    return {"solves_per_s": round(len(lat) / makespan, 3), "p50_s": round(_pct(lat, 50), 3),
            "p90_s": round(_pct(lat, 90), 3), "p99_s": round(_pct(lat, 99), 3),
            "mean_s": round(sum(lat) / len(lat), 3)}


def run_served(n_req: int, loads, budget_gb: float = 120.0, seed: int = 4,
               policy: str = "deadline"):
    """(see _run_served; policy may list several, comma-separated: the first
    is the line's `served`, the others are reported beside it)"""
    pols = [p for p in policy.split(",") if p]
    return _run_served(n_req, loads, budget_gb, seed, pols)


def _run_served(n_req: int, loads, budget_gb: float, seed: int, policies):
    """Served configuration c5: a Poisson stream of requests (seeded serve
    mix, axes log-uniform 48..384, steps 200..4000) through the C request
    loop (continuous batching under an HBM budget, deadline policy), against
    the one-at-a-time plain-solver queue (FIFO) on the same GPU.

    1. Every request queued at once through the one-at-a-time queue: each
       request's time alone (admission to result, set-up included), its
       probe record, and the capacity (solves/s) the loads refer to.
    2. Per load: Poisson arrivals at load x capacity through the served
       loop and through the one-at-a-time queue, both live; beside them the
       queue's latencies as they follow from the measured times alone (a
       single server in arrival order: start = max(arrival, previous
       finish)), for reference.
    While the server is idle (nothing queued or running) the client does not
    wait for the next arrival but moves the clock on: latencies are
    unchanged, and solves/s count the skipped time.
    Every served request's probes must equal its one-at-a-time probes."""
    from maxwell_solver_gb300.serve import Server
    from maxwell_solver_gb300.workloads import serve_mix

    specs = serve_mix(n_req, seed)
    budget = int(budget_gb * (1 << 30))

    def one_run(arrivals, one_at_a_time, policy=policies[0]):
        with Server(hbm_budget=budget, one_at_a_time=one_at_a_time, policy=policy) as srv:
            t0 = time.perf_counter()
            skipped = 0.0
            tickets = []
            for spec, at in zip(specs, arrivals):
                while True:
                    left = at - (time.perf_counter() - t0 + skipped)
                    if left <= 0:
                        break
                    st = srv.stats()
                    if st["queued"] == 0 and st["active"] == 0:
                        skipped += left  # idle: move the clock to the arrival
                        break
                    time.sleep(min(left, 0.02))
                tickets.append(srv.submit(spec, n_probes=8))
            res = [srv.result(t) for t in tickets]
            st = srv.stats()
        lat = [r["info"]["latency_s"] for r in res]
        slow = sorted(range(len(lat)), key=lambda i: -lat[i])[:3]
        out = {**_lat_summary(lat, st["elapsed_s"] + skipped),
               "slowest": [{"latency_s": round(lat[i], 3), "cells": specs[i].cells,
                            "steps": specs[i].steps} for i in slow],
               "Mcell_steps_per_s": round(st["cell_steps"] / (st["elapsed_s"] + skipped) / 1e6, 1),
               "peak_active": st["peak_active"],
               "peak_reserved_GB": round(st["peak_reserved_bytes"] / (1 << 30), 2),
               "completed": st["completed"], "failed": st["failed"],
               "seconds_run": round(time.perf_counter() - t0, 2),
               "seconds_skipped_idle": round(skipped, 2)}
        return out, res

    # 1. one at a time, all queued: times alone, capacity, reference records
    sat, base = one_run([0.0] * len(specs), True)
    alone = [r["info"]["finish_s"] - r["info"]["admit_s"] for r in base]
    capacity = len(specs) / sum(alone)
    ref = [r["probes"] for r in base]

    def fifo_model(arrivals):
        fin, lat = 0.0, []
        for at, t in zip(arrivals, alone):
            fin = max(at, fin) + t
            lat.append(fin - at)
        return _lat_summary(lat, fin - arrivals[0])

    rng = np.random.default_rng(seed + 1)
    gaps = rng.exponential(1.0, len(specs))
    points, same = [], True
    for load in loads:
        rate = load * capacity
        arrivals = [float(x) for x in np.cumsum(gaps / rate) - gaps[0] / rate]
        served, res = one_run(arrivals, False)
        same &= all(np.array_equal(r["probes"], p) for r, p in zip(res, ref))
        fifo = fifo_model(arrivals)
        pt = {"load": load, "rate_per_s": round(rate, 3), "served": served}
        for pol in policies[1:]:
            other, res_o = one_run(arrivals, False, pol)
            same &= all(np.array_equal(r["probes"], p) for r, p in zip(res_o, ref))
            pt[f"served_{pol}"] = other
        live, res_l = one_run(arrivals, True)
        same &= all(np.array_equal(r["probes"], p) for r, p in zip(res_l, ref))
        pt["one_at_a_time"] = live
        pt["one_at_a_time_model"] = fifo
        pt["served_p50_le_fifo"] = bool(served["p50_s"] <= live["p50_s"])
        pt["served_p99_le_fifo"] = bool(served["p99_s"] <= live["p99_s"])
        pt["speedup_solves_per_s"] = round(served["solves_per_s"] / live["solves_per_s"], 3)
        log(f"served load {load}: {json.dumps(pt)}")
        points.append(pt)
    return {
        "workload": f"c5: {len(specs)} requests (seed {seed}), cubic-ish axes log-U[48,384], "
                    "CPML 8..16, spheres (oblique TF/SF, mode 5) or layers (mode 1), "
                    "steps U[200,4000], 8 probes each; Poisson arrivals",
        "policy": policies[0], "hbm_budget_GB": budget_gb,
        "capacity_solves_per_s": round(capacity, 3), "one_at_a_time_saturated": sat,
        "loads": points, "identical_results": bool(same),
        "timing": "wall clock from each request's submission to its result on the host "
                  "(set-up on the device, all steps, probe readout), served and one at a "
                  "time both live; idle gaps skipped, see run_served",
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", choices=("ours", "reference"), default="ours")
    ap.add_argument("--workload", default="c3", choices=("c1", "c2", "c3"))
    ap.add_argument("--tune-cache", default="",
                    help="autotuner cache file to use (default: a fresh one per run)")
    ap.add_argument("--e2e-steps", type=int, default=0,
                    help="steps of the end-to-end solve (0: the configuration's)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-e2e", action="store_true", help="skip the end-to-end leg")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched (c4) leg")
    ap.add_argument("--no-coef-arrays", action="store_true",
                    help="skip the per-cell coefficient array leg")
    ap.add_argument("--batch-grids", type=int, default=256)
    ap.add_argument("--batch-only", action="store_true",
                    help="run only the batched leg, without its one-at-a-time baselines")
    ap.add_argument("--no-serve", action="store_true", help="skip the served (c5) leg")
    ap.add_argument("--serve-requests", type=int, default=100)
    ap.add_argument("--serve-loads", default="0.3,0.6,0.9,1.2",
                    help="offered loads, fractions of the measured batched capacity")
    ap.add_argument("--serve-only", action="store_true", help="run only the served leg")
    ap.add_argument("--serve-policy", default="deadline",
                    help="served order(s): deadline, srpt, bounded, hrrn; a comma-separated "
                         "list runs each (the first is the line's)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    # the reference arm runs on rank 0 alone; the other ranks leave at once
    # (a rank waiting in the process group would spin on a core the OpenMP
    # oracle's threads need)
    ranks = Ranks(join=args.impl != "reference")
    if args.batch_only:
        print(json.dumps({"batched": run_batched(args.batch_grids, batched_only=True)}), flush=True)
        return
    if args.serve_only:
        loads = [float(x) for x in args.serve_loads.split(",") if x]
        print(json.dumps({"served": run_served(args.serve_requests, loads,
                                               policy=args.serve_policy)}), flush=True)
        return
    if args.impl == "reference":
        out = run_reference(args, ranks)
        ranks.close()
    else:
        out = run_ours(args, ranks)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
