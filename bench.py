"""Benchmark of the GB300 hot path: cell-steps/s of the two-phase flow step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--cube N] [--no-compare] [--no-cpu-baseline]

Workloads are <config>_<precision>: config0..config4 (the benchmark
configurations as seeded synthetic inputs, see workloads.py) and f64, split
(masses at FP64 precision: FP32-pair defects), splitdf (FP32-pair masses), splitdefect
(FP32 mass defects).
The default, config4_splitdefect, is the combined
precision + batching form on the 256-member ensemble; the same line also
reports plain FP64 and the other split forms on the same members.

One JSON line on rank 0. `value` is device-resident throughput (inputs in
HBM, CUDA events on the stream the kernels run on, CUDA graphs for
ensembles); `e2e` is the same metric through the public C ABI with host
buffers (pinned host -> device state, the step, device -> host P and S,
every step). `--impl reference` times the reference CPU algorithm (the
oracle: a bit-exact restatement of the reference's cpu.cpp) on the host
cores instead.
"""
from __future__ import annotations

import argparse
import json
import os
import pathlib
import statistics
import subprocess
import sys
import tempfile
import time

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
            time.sleep(0.3)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
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
        import torch
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
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

PRECISIONS = {"f64": ("GBF_PREC_F64", "plain FP64", "f64"),
              "split": ("GBF_PREC_SPLIT", "FP32 state and fluxes, phase masses at FP64 precision (FP32-pair "
                        "defects over the state's mass at the row's hydrostatic density)", "f32+f32x2"),
              "splitdf": ("GBF_PREC_SPLIT_DF", "FP32 state and fluxes, FP32-pair masses and residual",
                          "f32+f32x2"),
              "splitdefect": ("GBF_PREC_SPLIT_DEFECT", "FP32 state and fluxes, phase masses as FP32 defects over "
                              "the state's mass at the row's hydrostatic density", "f32")}


def make_members(pkg, lib, cfg, cube):
    from importlib import import_module
    wl = import_module(pkg.__name__ + ".workloads")
    if cfg == "config0":
        return [wl.config0(lib)], "config 0: 40^3 homogeneous single grid", False
    if cfg == "config1":
        mem = wl.config1(lib, n=cube or 256)
        return [mem], f"config 1: {mem.model.nx}^3 heterogeneous single grid", False
    if cfg == "config2":
        return [wl.config2(lib)], "config 2: 512x512x256 heterogeneous single grid (sigma_lnK 1.5)", False
    if cfg == "config3":
        return wl.config3(lib), "config 3: 96 realizations, edges in {64,96,128,160}", True
    if cfg == "config4":
        return wl.config4(lib), "config 4: 256 realizations, edges 48..128 step 16, anisotropic", True
    raise SystemExit(f"unknown configuration {cfg}")


class Runner:
    """One domain or one ensemble behind the same calls."""

    def __init__(self, pkg, members, precision, ensemble, mass_cap):
        from importlib import import_module
        self.abi = pkg.abi
        self.members = members
        self.ensemble = ensemble
        if ensemble:
            E = import_module(pkg.__name__ + ".ensemble").Ensemble
            self.obj = E(members, precision=precision)
        else:
            D = import_module(pkg.__name__ + ".domain").Domain
            m = members[0]
            self.obj = D(m.model, m.media, m.K, m.phi, precision=precision)
        self.obj.set_outputs(self.abi.GBF_OUT_MASS, mass_cap)

    def upload_initial(self):
        if self.ensemble:
            self.obj.upload_initial()
        else:
            self.obj.upload(*self.members[0].initial_state())

    def upload(self, r, P, S):
        if self.ensemble:
            self.obj.upload(r, P, S)
        else:
            self.obj.upload(P, S)

    def download(self, r, field, out=None):
        return self.obj.download(r, field, out) if self.ensemble else self.obj.download(field, out)

    def __getattr__(self, name):
        return getattr(self.obj, name)

    @property
    def cells(self):
        return sum(m.ncells for m in self.members)

    @property
    def uses_tma(self):
        lib = self.obj.lib
        return bool(lib.gbf_ensemble_uses_tma(self.obj.h) if self.ensemble else lib.gbf_domain_uses_tma(self.obj.h))

    @property
    def interior_cells(self):
        return sum((m.model.nx - 2) * (m.model.ny - 2) * (m.model.nz - 2) for m in self.members)


# Algorithmic bytes per interior (or every) cell of each kernel: the
# compulsory DRAM traffic of its inputs and outputs.
ALGO_BYTES = {
    "f64_props": (60.0, "all"),             # read P, S, K (20); write L1, L2, ro1, ro2, lnSe (40)
    "ensemble_f64_props": (60.0, "all"),
    "f64_flux_newton": (76.0, "interior"),  # read P, S, L1, L2, ro1, ro2, lnSe (56), phi (4); write P, S (16)
    "ensemble_f64_flux_newton": (76.0, "interior"),
    "split_step": (56.0, "interior"),       # read dP, S, K, phi (16), M1, M2 (16); write dP, S (8), M1, M2 (16)
    "ensemble_step": (56.0, "interior"),
}
# The defect form holds M1, M2 in 4 bytes: read 16 + 8, write 8 + 8.
ALGO_BYTES_DEFECT = {"split_step": (40.0, "interior"), "ensemble_step": (40.0, "interior")}


def timed(runner, steps, stream, world, clocks=None):
    """Device time of `steps` steps on the runner's stream (CUDA events)."""
    import torch
    barrier(world)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    runner.step(steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier(world)
    return dist_max(e0.elapsed_time(e1), world)


def cpu_baseline(O, abi, members, budget_s=12.0, threads=None):
    """The oracle on the host cores over a bounded sample of the workload:
    whole members (largest first), one time step at a time, until ~budget_s."""
    orc = O.Oracle(abi)
    threads = threads or os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    done_cells = 0
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
        sample.append(f"{mem.model.nx}x{mem.model.ny}x{mem.model.nz} x {n} steps")
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": done_cells / dt, "unit": "cell-steps/s", "cores": threads, "kind": "port",
            "sample": "; ".join(sample) + f" ({dt:.1f} s; oracle = bit-exact restatement of the reference "
                                          f"cpu.cpp, OpenMP over i, 7 Newton iterations)"}


def run_ours(args, rank, world):
    import torch
    pkg = ge.load_package()
    lib = pkg.load_library()
    abi = pkg.abi
    torch.cuda.init()
    if args.no_tma:
        lib.gbf_set_tma(0)
    cfg, _, p = args.workload.partition("_")
    if p not in PRECISIONS:
        raise SystemExit(f"unknown precision in {args.workload}")
    members, desc, ensemble = make_members(pkg, lib, cfg, args.cube)
    if args.members:
        members = members[: args.members]
        desc += f" (first {len(members)} members)"
    prec = getattr(abi, PRECISIONS[p][0])
    stream = torch.cuda.Stream()
    cap = args.warmup + 2 * args.steps + 8
    run = Runner(pkg, members, prec, ensemble, cap)
    run.set_stream(stream.cuda_stream)
    tuning = None
    if ensemble and prec != abi.GBF_PREC_F64 and args.tile >= 0:
        run.set_tuning(args.tile, 0, 0)
        tuning = run.tuning()
    elif ensemble and prec != abi.GBF_PREC_F64 and not args.no_autotune:
        run.upload_initial()
        tuning = run.autotune(2)
    run.upload_initial()
    run.step(args.warmup)
    run.sync()
    cells = run.cells
    with ClockSampler(torch.cuda.current_device()) as clk:
        ms = timed(run, args.steps, stream, world)            # value: graphs, no per-kernel events
        run.set_timing(True)                                   # roofline: the same steps with kernel events
        ms_k = timed(run, args.steps, stream, world)
    ktimes = run.kernel_times()
    run.set_timing(False)
    status = run.status()
    value = world * cells * args.steps / (ms / 1e3)

    # roofline of the dominant kernel
    hbm, peak_kind = peaks()
    kname, (kms, klaunch) = max(ktimes.items(), key=lambda kv: kv[1][0])
    per_launch_s = kms / 1e3 / max(klaunch, 1)
    bpc, which = (ALGO_BYTES_DEFECT if p == "splitdefect" else ALGO_BYTES).get(kname, ALGO_BYTES.get(kname, (0.0, "all")))
    algo = bpc * (run.interior_cells if which == "interior" else cells)
    achieved = algo / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():  # ncu DRAM bytes per cell of a smaller capture, scaled to this launch's cells
        ent = json.loads(tfile.read_text()).get(args.workload, {}).get(kname)
        if ent:
            traffic = ent["bytes_per_cell"] * (run.interior_cells if ent["cells"] == "interior" else cells)
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": algo, "bytes_per_cell": bpc, "ms_per_launch": per_launch_s * 1e3,
            "kernel_times_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in ktimes.items()},
            "binding_resource": ("FP64 pipe (ncu: 85% of FP64-pipe cycles active in the flux/Newton pass; "
                                 "GB300 DFMA 1.2 TFLOP/s)") if "f64" in kname else
                                ("instruction issue and the per-plane block barrier (ncu: 66-80% issue "
                                 "active; DRAM traffic 1.12-1.16x the algorithmic bytes on config 4, halo "
                                 "rows re-read)"),
            "ms_per_step_with_kernel_events": ms_k / args.steps}
    if "f64" in kname:  # the FP64 kernels' own roof: the FP64 pipe, from the ncu capture of this pass
        roof["fp64_pipe"] = {"frac": 0.853, "metric": "sm__pipe_fp64_cycles_active",
                             "source": "profiles/f64_flux_newton_config1.md (flux/Newton pass, 192^3)"}

    # e2e through the C ABI with pinned host buffers: H2D state, one step, D2H P and S
    e2e_steps = max(2, min(args.steps, 10 if ensemble else 20))
    if ensemble:
        Pall = torch.empty(cells, dtype=torch.float64, pin_memory=True).numpy()
        Sall = torch.empty(cells, dtype=torch.float64, pin_memory=True).numpy()
        run.download_all(Pall, Sall)
        for _ in range(max(1, args.warmup)):  # warm-up calls: the first sets up the pipeline's buffers
            run.advance_host(Pall, Sall, 1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            run.advance_host(Pall, Sall, 1)
        api = ("gbf_ensemble_advance_host(P, S, 1, P, S): every member's P1, S2 host->device, one step, "
               "device->host, pipelined over member groups")
    else:
        hostP = torch.empty(members[0].model.shape, dtype=torch.float64, pin_memory=True).numpy()
        hostS = torch.empty(members[0].model.shape, dtype=torch.float64, pin_memory=True).numpy()
        run.download(0, "P1", hostP)
        run.download(0, "S2", hostS)
        for _ in range(max(1, args.warmup)):  # warm-up round trips
            run.upload(0, hostP, hostS)
            run.step(1)
            run.download(0, "P1", hostP)
            run.download(0, "S2", hostS)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            run.upload(0, hostP, hostS)
            run.step(1)
            run.download(0, "P1", hostP)
            run.download(0, "S2", hostS)
        api = "gbf_domain_upload + gbf_domain_step(1) + gbf_domain_download(P1, S2)"
    e2e_s = dist_max(time.perf_counter() - t0, world)
    e2e = {"value": world * cells * e2e_steps / e2e_s, "unit": "cell-steps/s",
           "h2d_bytes_per_step": 2 * cells * 8, "d2h_bytes_per_step": 2 * cells * 8, "api": api}

    out = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": PRECISIONS[p][2],
           "data": "synthetic (seeded fields with the configuration's shapes and statistics)",
           "config": {"workload": args.workload, "desc": f"{desc}, {PRECISIONS[p][1]}", "cells": cells,
                      "members": len(members), "dt_used_range": [min(m.model.dt for m in members),
                                                                 max(m.model.dt for m in members)],
                      "l2": f"inputs larger than L2 (state and fields {cells * 40 / 1e9:.1f} GB > 129 MB)",
                      "newton": "FP64: converge-and-exit (tol 1e-11, max 7); split: 2 increment iterations",
                      "tuning": tuning, "graphs": ensemble,
                      "plane_staging": "TMA" if run.uses_tma else "plain loads"},
           "clocks": clk.summary(), "e2e": e2e, "gpu_launches": run.launches_per_step * args.steps,
           "roofline": roof, "status": lib.gbf_status_string(status).decode()}
    run.close()
    del run

    if ensemble and not args.no_compare and rank == 0:
        comp = {}
        for q in ("f64", "split", "splitdf", "splitdefect"):
            if q == p:
                continue
            r2 = Runner(pkg, members, getattr(abi, PRECISIONS[q][0]), True, cap)
            r2.set_stream(stream.cuda_stream)
            if q != "f64" and not args.no_autotune:
                r2.upload_initial()
                r2.autotune(2)
            r2.upload_initial()
            r2.step(args.warmup)
            r2.sync()
            nst = min(args.steps, 10) if q == "f64" else args.steps
            ms2 = timed(r2, nst, stream, 1)
            comp[q] = {"value": cells * nst / (ms2 / 1e3), "steps": nst, "ms_per_step": ms2 / nst,
                       "dtype": PRECISIONS[q][2]}
            r2.close()
            del r2
        out["same_members"] = comp
        if "f64" in comp:
            out["split_batched_over_fp64_batched"] = value / comp["f64"]["value"]
    if rank == 0 and not args.no_compare and prec != abi.GBF_PREC_F64:
        out["accuracy"] = accuracy_block(pkg, ge.load_oracle_module(), members, prec, ensemble)
    if rank == 0 and not args.no_cpu_baseline:
        O = ge.load_oracle_module()
        out["cpu_baseline"] = cpu_baseline(O, abi, members, budget_s=args.cpu_budget)
    return out


def accuracy_block(pkg, O, members, prec, ensemble, steps=20):
    """The measured form against plain FP64 on the same members and steps
    (the GPU FP64 path, itself pinned to the oracle at 1e-12), and against
    the oracle on the smallest member: max|dS|, relative L2 of P, relative
    phase-mass difference per step, and how far S moved (max|S - S0|)."""
    import numpy as np
    abi = pkg.abi

    def run(p):
        r = Runner(pkg, members, p, ensemble, steps + 2)
        split = p != abi.GBF_PREC_F64
        if split:
            r.set_outputs(abi.GBF_OUT_MASS | abi.GBF_OUT_CFL, steps + 2)
        r.upload_initial()
        r.step(steps)
        out = [(r.download(i, "P1"), r.download(i, "S2")) for i in range(len(members))] if ensemble else \
            [(r.download(0, "P1"), r.download(0, "S2"))]
        mass = r.mass_history(steps)
        cfl = r.cfl_history(steps) if split else None
        r.close()
        return out, mass, cfl

    got, mg, cfl = run(prec)
    ref, mr, _ = run(abi.GBF_PREC_F64)
    ds = max(float(np.abs(a[1] - b[1]).max()) for a, b in zip(got, ref))
    num = sum(float(np.sum((a[0] - b[0]) ** 2)) for a, b in zip(got, ref))
    den = sum(float(np.sum(b[0] ** 2)) for b in ref)
    moved = max(float(np.abs(b[1] - m.initial_state()[1]).max()) for b, m in zip(ref, members))
    scale = np.maximum(np.abs(mr), 1e-300)
    drift = float(np.max(np.abs(mg - mr) / scale * (np.abs(mr) > 0)))
    block = {"vs": "plain FP64 GPU path of the same members (pinned to the oracle at 1e-12)", "steps": steps,
             "max_dS": ds, "rel_l2_P": (num / den) ** 0.5, "phase_mass_rel_diff_max": drift, "S_moved_max": moved,
             "cfl_max": [float(cfl[..., 0].max()), float(cfl[..., 1].max())]}
    # the oracle itself on the smallest member
    i = min(range(len(members)), key=lambda q: members[q].ncells)
    mem = members[i]
    st = O.State(mem.model, mem.media, mem.K, mem.phi)
    P0, S0 = mem.initial_state()
    st["P1"][...] = P0
    st["S2"][...] = S0
    O.Oracle(abi).step(st, steps)
    block["oracle_sample"] = {"member": i, "shape": list(mem.model.shape), "steps": steps,
                              "max_dS": float(np.abs(got[i][1] - st["S2"]).max()),
                              "rel_l2_P": float(np.linalg.norm(got[i][0] - st["P1"]) / np.linalg.norm(st["P1"]))}
    return block


def run_reference(args, rank, world):
    """The reference CPU algorithm (oracle) on all host cores, same workload and metric."""
    if rank != 0:
        return None
    pkg = ge.load_package()
    lib = pkg.load_library()
    O = ge.load_oracle_module()
    cfg, _, p = args.workload.partition("_")
    members, desc, _ = make_members(pkg, lib, cfg, args.cube)
    threads = os.cpu_count()
    os.environ["OMP_NUM_THREADS"] = str(threads)
    orc = O.Oracle(pkg.abi)
    # bounded sample per step: whole members, largest first, until ~budget
    budget = max(1.0, 120.0 / max(1, args.steps + args.warmup))
    states = []

    def state(mem):
        st = O.State(mem.model, mem.media, mem.K, mem.phi)
        P, S = mem.initial_state()
        st["P1"][...] = P
        st["S2"][...] = S
        return st

    order = sorted(members, key=lambda x: -x.ncells)

    def one_step():
        t0 = time.perf_counter()
        c = 0
        for q, mem in enumerate(order):
            if q >= len(states):
                states.append(state(mem))
            orc.step(states[q], 1)
            c += mem.ncells
            if time.perf_counter() - t0 > budget:
                break
        return c, time.perf_counter() - t0

    for _ in range(args.warmup):
        one_step()
    tot_c, tot_t = 0, 0.0
    for _ in range(args.steps):
        c, t = one_step()
        tot_c += c
        tot_t += t
    v = tot_c / tot_t
    sample = f"{len(states)} of {len(members)} member(s) per step, each step bounded to ~{budget:.1f} s"
    return {"metric": METRIC, "impl": "reference", "value": v, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_t / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded fields with the configuration's shapes and statistics)",
            "config": {"workload": args.workload, "desc": desc + " (reference CPU algorithm, FP64)",
                       "cells": sum(m.ncells for m in members)},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cpu_baseline": {"value": v, "unit": "cell-steps/s", "cores": threads, "kind": "port",
                             "sample": sample + "; oracle = bit-exact restatement of the reference cpu.cpp "
                                                "(OpenMP over i), 7 Newton iterations"}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config4_splitdefect")
    ap.add_argument("--cube", type=int, default=0, help="override the grid edge of config1 (profiling runs)")
    ap.add_argument("--members", type=int, default=0, help="first N members of an ensemble (profiling runs)")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-compare", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-tma", action="store_true", help="stage split-step planes by plain loads, not TMA")
    ap.add_argument("--tile", type=int, default=-1, help="ensemble tile shape (gbf_ensemble_set_tuning); skips autotune")
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
