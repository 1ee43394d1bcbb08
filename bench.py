"""Benchmark of the GB300 hot path: cell-steps/s of the two-phase flow step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--cube N]

One JSON line on rank 0. `value` is device-resident throughput (inputs in
HBM, CUDA events on the stream the kernels run on); `e2e` is the same metric
through the public C ABI with host buffers (pinned host -> device copy of the
state, the step, device -> host copy of P and S, every step). `--impl
reference` times the reference CPU algorithm (the oracle: a bit-exact
restatement of the reference's cpu.cpp) on the host cores instead.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
import pathlib

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
import __graft_entry__ as ge  # noqa: E402

METRIC = "cell-steps/s on 1 GB300: FP32/FP64-split batched vs plain FP64, max|dS|<=1e-5"
PEAKS = ROOT / "MEASURED_PEAKS.json"
FALLBACK_HBM_GBS = 6800.0


def peaks():
    if PEAKS.exists():
        p = json.loads(PEAKS.read_text())
        return float(p["hbm_gbs"]), "measured"
    return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.TemporaryFile(mode="w+")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.f:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.seek(0)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.f.read().strip().splitlines():
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for n, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        import torch
        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend)
        if torch.cuda.is_available():
            torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    return rank, world


def dist_max(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------------ workloads

PRECISIONS = {"f64": ("GBF_PREC_F64", "plain FP64"),
              "split": ("GBF_PREC_SPLIT", "FP32 state and fluxes, FP64 masses and residual"),
              "splitdf": ("GBF_PREC_SPLIT_DF", "FP32 state and fluxes, FP32-pair masses and residual")}


def make_workload(pkg, lib, name, cube):
    from importlib import import_module
    wl = import_module(pkg.__name__ + ".workloads")
    cfg, _, p = name.partition("_")
    if p not in PRECISIONS:
        raise SystemExit(f"unknown workload {name}")
    prec = getattr(pkg.abi, PRECISIONS[p][0])
    if cfg == "config1":
        mem = wl.config1(lib, n=cube or 256)
        desc = f"config 1: {mem.model.nx}^3 heterogeneous single grid"
    elif cfg == "config0":
        mem = wl.config0(lib)
        desc = "config 0: 40^3 homogeneous"
    elif cfg == "config2":
        mem = wl.config2(lib)
        desc = "config 2: 512x512x256 heterogeneous single grid (sigma_lnK 1.5)"
    else:
        raise SystemExit(f"unknown workload {name}")
    return {"members": [mem], "precision": prec, "desc": f"{desc}, {PRECISIONS[p][1]}"}


# Algorithmic bytes per cell of each kernel (compulsory DRAM traffic of its
# inputs and outputs).
ALGO_BYTES = {
    "f64_props": 60.0,        # read P, S (16), K (4) = 20; write L1, L2, ro1, ro2, lnSe (40)
    "f64_flux_newton": 76.0,  # read P, S, L1, L2, ro1, ro2, lnSe (56), phi (4); write P, S (16)
    "split_step": 56.0,       # read dP, S, K, phi (16), M1, M2 (16); write dP, S (8), M1, M2 (16)
}
KERNEL_CELLS = {"f64_props": "all", "f64_flux_newton": "interior", "split_step": "interior"}


def cells_of(m, which):
    if which == "all":
        return m.nx * m.ny * m.nz
    return (m.nx - 2) * (m.ny - 2) * (m.nz - 2)


def cpu_baseline(O, abi, members, budget_s=12.0, threads=None):
    """The oracle on the host cores over a bounded sample of the workload:
    whole members (largest first), one time step at a time, until ~budget_s."""
    orc = O.Oracle(abi)
    threads = threads or os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    done_cells = 0
    steps = 0
    t0 = time.perf_counter()
    sample = []
    for mem in sorted(members, key=lambda x: -x.ncells):
        st = O.State(mem.model, mem.media, mem.K, mem.phi)
        P, S = mem.initial_state()
        st["P1"][...] = P
        st["S2"][...] = S
        n = 0
        while time.perf_counter() - t0 < budget_s or n == 0:
            orc.step(st, 1)
            done_cells += mem.ncells
            n += 1
            if n >= 1000:
                break
        steps += n
        sample.append(f"{mem.model.nx}x{mem.model.ny}x{mem.model.nz} x {n} steps")
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": done_cells / dt, "unit": "cell-steps/s", "cores": threads, "kind": "port",
            "sample": "; ".join(sample) + f" ({dt:.1f} s, oracle = bit-exact restatement of cpu.cpp, "
                                          f"OpenMP over i, 7 Newton iterations)"}


def run_ours(args, rank, world):
    import torch
    pkg = ge.load_package()
    lib = pkg.load_library()
    abi = pkg.abi
    from importlib import import_module
    Domain = import_module(pkg.__name__ + ".domain").Domain
    torch.cuda.init()
    wl = make_workload(pkg, lib, args.workload, args.cube)
    mems = wl["members"]
    assert len(mems) == 1, "single-grid workloads only in this version"
    mem = mems[0]
    m = mem.model
    dom = Domain(m, mem.media, mem.K, mem.phi, precision=wl["precision"])
    dom.set_outputs(abi.GBF_OUT_MASS, args.warmup + args.steps + 8)
    P0, S0 = mem.initial_state()
    dom.upload(P0, S0)
    stream = torch.cuda.Stream()
    dom.set_stream(stream.cuda_stream)
    dom.step(args.warmup)
    dom.sync()
    barrier(world)
    torch.cuda.synchronize()
    dom.set_timing(True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(torch.cuda.current_device()) as clk:
        e0.record(stream)
        dom.step(args.steps)
        e1.record(stream)
        e1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    ms = e0.elapsed_time(e1)
    ktimes = dom.kernel_times()
    dom.set_timing(False)
    status = dom.status()
    ms_max = dist_max(ms, world)
    cells = mem.ncells
    value = world * cells * args.steps / (ms_max / 1e3)

    # e2e through the C ABI with pinned host buffers: H2D state, step, D2H P and S
    Ph = torch.empty(m.shape, dtype=torch.float64, pin_memory=True).numpy()
    Sh = torch.empty(m.shape, dtype=torch.float64, pin_memory=True).numpy()
    Ph[...] = dom.download("P1")
    Sh[...] = dom.download("S2")
    e2e_steps = max(3, min(args.steps, 20))
    dom.upload(Ph, Sh)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        dom.upload(Ph, Sh)
        dom.step(1)
        dom.download("P1", Ph)
        dom.download("S2", Sh)
    e2e_s = dist_max(time.perf_counter() - t0, world)
    e2e = {"value": world * cells * e2e_steps / e2e_s, "unit": "cell-steps/s",
           "h2d_bytes_per_step": 2 * cells * 8, "d2h_bytes_per_step": 2 * cells * 8,
           "api": "gbf_domain_upload + gbf_domain_step(1) + gbf_domain_download(P1, S2)"}

    # roofline of the dominant kernel
    hbm, peak_kind = peaks()
    dom_k = max(ktimes.items(), key=lambda kv: kv[1][0])
    kname, (kms, klaunch) = dom_k
    per_launch_s = kms / 1e3 / max(klaunch, 1)
    algo = ALGO_BYTES.get(kname, 0.0) * cells_of(m, KERNEL_CELLS.get(kname, "all"))
    achieved = algo / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():
        tj = json.loads(tfile.read_text())
        ent = tj.get(args.workload, {}).get(kname)
        if ent:
            traffic = ent["bytes_per_launch"]
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": algo, "ms_per_launch": per_launch_s * 1e3,
            "kernel_times_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in ktimes.items()}}
    mass = dom.mass_history(args.warmup + args.steps)
    out = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None,
           "dtype": {abi.GBF_PREC_F64: "f64", abi.GBF_PREC_SPLIT: "f32+f64",
                     abi.GBF_PREC_SPLIT_DF: "f32+f32x2"}[wl["precision"]],
           "data": "synthetic (seeded fields with the configuration's shapes and statistics)",
           "config": {"workload": args.workload, "desc": wl["desc"], "cells": cells,
                      "grid": [m.nx, m.ny, m.nz], "dt_used": m.dt,
                      "l2": "inputs larger than L2 (state+fields %.1f GB > 129 MB)" % (cells * 100 / 1e9),
                      "newton_tol": m.newton_tol},
           "clocks": clk.summary(), "e2e": e2e, "gpu_launches": dom.launches_per_step * args.steps,
           "roofline": roof, "status": lib.gbf_status_string(status).decode(),
           "phase_mass_last": mass[-1].tolist() if len(mass) else None}
    if rank == 0 and not args.no_cpu_baseline:
        O = ge.load_oracle_module()
        out["cpu_baseline"] = cpu_baseline(O, abi, mems, budget_s=args.cpu_budget)
    dom.close()
    return out


def run_reference(args, rank, world):
    """The reference CPU algorithm (oracle) on all host cores, same workload and metric."""
    if rank != 0:
        return None
    pkg = ge.load_package()
    lib = pkg.load_library()
    O = ge.load_oracle_module()
    wl = make_workload(pkg, lib, args.workload, args.cube)
    mems = wl["members"]
    threads = os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    orc = O.Oracle(pkg.abi)
    states = []
    for mem in mems:
        st = O.State(mem.model, mem.media, mem.K, mem.phi)
        P, S = mem.initial_state()
        st["P1"][...] = P
        st["S2"][...] = S
        states.append(st)
    # bounded sample per step: whole members until ~budget per step
    budget = max(1.0, 120.0 / max(1, args.steps + args.warmup))

    def one_step():
        t0 = time.perf_counter()
        cells = 0
        for st in states:
            orc.step(st, 1)
            cells += st.model.nx * st.model.ny * st.model.nz
            if time.perf_counter() - t0 > budget:
                break
        return cells, time.perf_counter() - t0

    for _ in range(args.warmup):
        one_step()
    tot_c, tot_t = 0, 0.0
    for _ in range(args.steps):
        c, t = one_step()
        tot_c += c
        tot_t += t
    v = tot_c / tot_t
    sample = f"{len(states)} member(s), whole steps bounded to ~{budget:.1f} s each"
    return {"metric": METRIC, "impl": "reference", "value": v, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded fields with the configuration's shapes and statistics)",
            "config": {"workload": args.workload, "desc": wl["desc"] + " (CPU oracle)",
                       "cells": sum(s.model.nx * s.model.ny * s.model.nz for s in states)},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                             "sample": sample + "; oracle = bit-exact restatement of the reference cpu.cpp "
                                                "(OpenMP over i), 7 Newton iterations"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config1_f64")
    ap.add_argument("--cube", type=int, default=0, help="override the grid edge (profiling runs)")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    if args.warmup < 3 and args.impl == "ours" and not args.cube:
        args.warmup = 3
    rank, world = dist_setup()
    out = run_reference(args, rank, world) if args.impl == "reference" else run_ours(args, rank, world)
    if rank == 0 and out is not None:
        print(json.dumps(out))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
