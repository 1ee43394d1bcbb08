"""Benchmark of the GB300 hot path: cell-steps/s of the two-phase flow step.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload NAME] [--cube N] [--no-compare] [--no-cpu-baseline]

Workloads are <config>_<form>: config0..config4 (the benchmark configurations
as seeded synthetic inputs, see workloads.py) and the forms f64 (plain FP64),
split (FP32 state and fluxes, phase masses at FP64 precision as FP32-pair
defects, one residual-correction Newton step per cell), splitdf (FP32-pair
masses), splitdefect (FP32 mass defects, no correction step); and
config1_dropin / config1_dropinsplit, config 1's grid through the reference's
own host function set (defines.h: the five calls of time_step_function) in
fused FP64 mode / split mode.
The default, config4_split, is the combined precision + batching form on the
256-member ensemble; the same line also reports plain FP64 and the other split
forms on the same members.

One JSON line on rank 0. `value` is device-resident throughput (inputs in
HBM, CUDA events on the stream the kernels run on, CUDA graphs for
ensembles); `e2e` is the same metric through the public C ABI with host
buffers (pinned host -> device state, the step, device -> host P and S,
every step). `--impl reference` times the reference CPU algorithm (the
oracle: a bit-exact restatement of the reference's cpu.cpp) on the host
cores instead, on inputs made by libgbf_inputs.so (libgbflow is not loaded).

Under torchrun (N ranks) an ensemble workload is N times the configuration's
members (the same parameter and field streams, continued) and rank r advances
members r, r + N, ...: per-GPU work stays that of the configuration ("weak");
single grids run one replica per rank.
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


def _dist_reduce(x: float, world: int, op):
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=op)
    return float(t.item())


def dist_max(x: float, world: int) -> float:
    import torch.distributed as dist
    return x if world == 1 else _dist_reduce(x, world, dist.ReduceOp.MAX)


def dist_sum(x: float, world: int) -> float:
    import torch.distributed as dist
    return x if world == 1 else _dist_reduce(x, world, dist.ReduceOp.SUM)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ------------------------------------------------------------------ workloads

PRECISIONS = {"f64": ("GBF_PREC_F64", "plain FP64", "f64"),
              "split": ("GBF_PREC_SPLIT", "FP32 state and fluxes, phase masses at FP64 precision (FP32-pair "
                        "defects over the state's mass at the row's hydrostatic density), one residual-"
                        "correction Newton step per cell with the residual in FP32 pairs", "f32+f32x2"),
              "splitdf": ("GBF_PREC_SPLIT_DF", "FP32 state and fluxes, FP32-pair masses and residual",
                          "f32+f32x2"),
              "splitdefect": ("GBF_PREC_SPLIT_DEFECT", "FP32 state and fluxes, phase masses as FP32 defects over "
                              "the state's mass at the row's hydrostatic density, no correction step", "f32"),
              "dropin": ("GBF_PREC_F64", "plain FP64 through the reference's host function set (defines.h), "
                         "fused mode", "f64"),
              "dropinsplit": ("GBF_PREC_SPLIT", "the split form (FP32 state and fluxes, phase masses at FP64 "
                              "precision, one residual-correction Newton step per cell) through the reference's "
                              "host function set (defines.h), split mode", "f32+f32x2")}
DROPIN_MODES = {"dropin": 1, "dropinsplit": 2}  # gbf_dropin_set_mode: fused FP64, split
ENSEMBLE_BASE = {"config3": 96, "config4": 256}
DESC = {"config0": "config 0: 40^3 homogeneous single grid",
        "config1": "config 1: {n}^3 heterogeneous single grid",
        "config1_dropin": "config 1's {n}^3 grid in the reference's media-table physics (Dirichlet patch, "
                          "reference boundary rules: all that the defines.h calls express)",
        "config2": "config 2: 512x512x256 heterogeneous single grid (sigma_lnK 1.5)",
        "config3": "config 3: {m} realizations, edges in {{64,96,128,160}}",
        "config4": "config 4: {m} realizations, edges 48..128 step 16, anisotropic"}


class Workload:
    """The workload of a --workload name: this rank's members, and the shape
    of the whole job (all ranks) from the members' parameters alone."""

    def __init__(self, pkg, lib, name, cube, rank, world, limit=0):
        from importlib import import_module
        self.wl = wl = import_module(pkg.__name__ + ".workloads")
        cfg, _, form = name.partition("_")
        if form not in PRECISIONS:
            raise SystemExit(f"unknown form in {name}")
        self.name, self.cfg, self.form = name, cfg, form
        self.ensemble = cfg in ENSEMBLE_BASE
        if form in DROPIN_MODES and cfg != "config1":
            raise SystemExit("the drop-in forms run config 1's grid only (config1_dropin, config1_dropinsplit)")
        n = cube or 256
        if self.ensemble:
            specs = (wl.config3_specs if cfg == "config3" else wl.config4_specs)(ENSEMBLE_BASE[cfg] * world)
            if limit:
                specs = [s for s in specs if s["index"] % ENSEMBLE_BASE[cfg] < limit]
            self.members_all = len(specs)
            self.cells_all = sum(wl.spec_cells(s) for s in specs)
            self.members = [wl.build_member(lib, s) for s in wl.shard(specs, rank, world)]
            self.desc = DESC[cfg].format(m=self.members_all)
            self.partition = (f"members r::{world} of {self.members_all} on rank r (weak scaling: "
                              f"{ENSEMBLE_BASE[cfg] if not limit else limit} members' worth per GPU)")
        else:
            if cfg == "config0":
                mem = wl.config0(lib)
            elif cfg == "config1":
                mem = wl.config1_dropin(lib, n=n) if form in DROPIN_MODES else wl.config1(lib, n=n)
            elif cfg == "config2":
                mem = wl.config2(lib)
            else:
                raise SystemExit(f"unknown configuration {cfg}")
            self.members = [mem]
            self.members_all = world
            self.cells_all = world * mem.ncells
            self.desc = DESC["config1_dropin" if form in DROPIN_MODES else cfg].format(n=n)
            self.partition = "replicas: one grid per rank" if world > 1 else "one grid"

    @property
    def cells(self):
        return sum(m.ncells for m in self.members)

    @property
    def interior_cells(self):
        return sum((m.model.nx - 2) * (m.model.ny - 2) * (m.model.nz - 2) for m in self.members)

    def config(self):
        """The `config` of the JSON line: the workload, identical in both arms."""
        gb = self.cells_all * 32 / 1e9
        return {"workload": self.name, "desc": self.desc, "cells": self.cells_all, "members": self.members_all,
                "form": PRECISIONS[self.form][1], "partition": self.partition,
                "l2": (f"inputs larger than L2 (state and fields >= {gb:.1f} GB > 129 MB)" if gb > 0.129 else
                       f"inputs smaller than L2 ({gb:.3f} GB): a profiling or test case")}


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
    def uses_tma(self):
        lib = self.obj.lib
        return bool(lib.gbf_ensemble_uses_tma(self.obj.h) if self.ensemble else lib.gbf_domain_uses_tma(self.obj.h))


class DropinRunner:
    """Config 1's grid through the reference's host function set, called like
    main.cpp: device_memory_alloc, load_data_to_device(_int), then per step
    time_step_function's five calls (main.cpp:83-94) in fused mode (1) or
    split mode (2)."""

    def __init__(self, pkg, member, mode=1):
        import ctypes
        from importlib import import_module
        self.abi = pkg.abi
        self.dp = dp = import_module(pkg.__name__ + ".dropin")
        self.mem = member
        self.di = dp.DropIn()
        self.di.set_mode(mode)
        m = member.model
        self.c = dp.consts_from_model(m)
        self.H = dp.PtrArrays()
        self.D = dp.PtrArrays()
        self.buf = ctypes.c_void_p()
        self.di.f["device_memory_alloc"](ctypes.byref(self.D), ctypes.byref(self.buf), m.nx, self.c)
        self.t = 0.0
        self.lib = self.di.lib
        status = self.lib.gbf_last_status()
        if status:
            raise RuntimeError(f"device_memory_alloc: {self.lib.gbf_status_string(status).decode()}")

    def upload(self, P, S):
        f, c = self.di.f, self.c
        f["load_data_to_device"](P.ctypes.data, self.D.P1, c.NX, c)
        f["load_data_to_device"](S.ctypes.data, self.D.S2, c.NX, c)

    def upload_initial(self):
        P, S = self.mem.initial_state()
        self.upload(P, S)
        media = np.zeros(self.mem.model.shape, np.int32) if self.mem.media is None else self.mem.media
        self.di.f["load_data_to_device_int"](np.ascontiguousarray(media, np.int32).ctypes.data, self.D.media,
                                             self.c.NX, self.c)
        self.t = 0.0

    def step(self, n=1):
        for _ in range(n):
            self.t += self.c.dt
            self.di.time_step(self.H, self.D, self.c, self.t)

    def download(self, field, out):
        self.di.f["load_data_to_host"](out.ctypes.data, getattr(self.D, field), self.c.NX, self.c)
        return out

    @property
    def handle(self):
        return self.di.domain(self.D.P1)

    def set_timing(self, on):
        h = self.handle
        if h:
            self.lib.gbf_domain_set_timing(h, int(on))

    def kernel_times(self):
        n = self.lib.gbf_kernel_kinds()
        ms = np.zeros(n, np.float64)
        cnt = np.zeros(n, np.int32)
        self.lib.gbf_domain_kernel_times(self.handle, ms.ctypes.data, cnt.ctypes.data, n)
        return {self.lib.gbf_kernel_name(k).decode(): (float(ms[k]), int(cnt[k])) for k in range(n) if cnt[k]}

    def status(self):
        h = self.handle
        return self.lib.gbf_domain_status(h) if h else self.lib.gbf_last_status()

    @property
    def uses_tma(self):
        h = self.handle
        return bool(h and self.lib.gbf_domain_uses_tma(h))

    def sync(self):
        import torch
        torch.cuda.synchronize()

    def close(self):
        if self.D.P1:
            self.di.f["device_memory_free"](self.D, self.buf)
            self.D.P1 = None


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
# The drop-in's media-table grid reads an int media index instead of K, phi (props: P, S, media;
# flux/Newton: no phi read).
# Split mode: read dP, S (8), media (4), M1, M2 (16); write dP, S (8), M1, M2 (16).
ALGO_BYTES_DROPIN = {"f64_props": (60.0, "all"), "f64_flux_newton": (72.0, "interior"),
                     "split_step": (52.0, "interior")}


def timed(runner, steps, stream, world):
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


# --------------------------------------------------- reference CPU algorithm

def reference_cpu_run(O, abi, members, steps, warmup, step_budget_s):
    """The reference CPU algorithm (the oracle: a bit-exact restatement of
    cpu.cpp, 7 Newton iterations, OpenMP over i) on all host cores. Each step
    advances whole members, largest first, until the step's time budget is
    spent (every member at least once per step counted); `steps` timed steps
    after `warmup` untimed ones. The same measurement serves the reference arm
    and the repo arm's cpu_baseline."""
    threads = os.cpu_count() or 1
    os.environ["OMP_NUM_THREADS"] = str(threads)
    orc = O.Oracle(abi)
    order = sorted(members, key=lambda x: -x.ncells)
    states = []

    def state(mem):
        st = O.State(mem.model, mem.media, mem.K, mem.phi)
        P, S = mem.initial_state()
        st["P1"][...] = P
        st["S2"][...] = S
        return st

    def one_step():
        t0 = time.perf_counter()
        c = 0
        for q, mem in enumerate(order):
            if q >= len(states):
                states.append(state(mem))
            orc.step(states[q], 1)
            c += mem.ncells
            if time.perf_counter() - t0 > step_budget_s:
                break
        return c, time.perf_counter() - t0

    for _ in range(warmup):
        one_step()
    tot_c, tot_t = 0, 0.0
    for _ in range(steps):
        c, t = one_step()
        tot_c += c
        tot_t += t
    v = tot_c / tot_t
    sample = (f"{len(states)} of {len(members)} member(s) per step (largest first), each step bounded to "
              f"~{step_budget_s:.1f} s, {steps} timed step(s) after {warmup}; oracle = bit-exact restatement of "
              f"the reference cpu.cpp (OpenMP over i), 7 Newton iterations")
    return {"value": v, "unit": "cell-steps/s", "cores": threads, "kind": "port", "sample": sample,
            "seconds": tot_t}


def step_budget(args):
    return max(1.0, 120.0 / max(1, args.steps + args.warmup))


# ------------------------------------------------------------------- our arm

def link_bandwidth(torch, nbytes=1 << 30, reps=3):
    """Pinned host <-> device copy rates (GB/s), each direction alone and both
    at once: the best of `reps` timed copies after one untimed round of each
    (the first use of a stream or buffer carries one-off costs)."""
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h2 = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()

    def h2d():
        d.copy_(h, non_blocking=True)

    def d2h():
        h.copy_(d, non_blocking=True)

    def both():
        with torch.cuda.stream(s1):
            d.copy_(h, non_blocking=True)
        with torch.cuda.stream(s2):
            h2.copy_(d2, non_blocking=True)

    best = {}
    for name, f in (("h2d", h2d), ("d2h", d2h), ("both", both)):
        f()
        torch.cuda.synchronize()
        t = []
        for _ in range(reps):
            t0 = time.perf_counter()
            f()
            torch.cuda.synchronize()
            t.append(time.perf_counter() - t0)
        best[name] = min(t)
    del h, h2, d, d2
    return {"h2d_gbs": nbytes / best["h2d"] / 1e9, "d2h_gbs": nbytes / best["d2h"] / 1e9,
            "both_gbs": 2 * nbytes / best["both"] / 1e9}


def run_ours(args, rank, world):
    import torch
    pkg = ge.load_package()
    lib = pkg.load_library()
    abi = pkg.abi
    torch.cuda.init()
    if args.no_tma:
        lib.gbf_set_tma(0)
    W = Workload(pkg, lib, args.workload, args.cube, rank, world, args.members)
    members, ensemble, p = W.members, W.ensemble, W.form
    prec = getattr(abi, PRECISIONS[p][0])
    cap = args.warmup + 2 * args.steps + 8
    tuning = None
    if p in DROPIN_MODES:
        stream = torch.cuda.default_stream()  # the drop-in runs on the legacy default stream, like gpu.cu
        run = DropinRunner(pkg, members[0], DROPIN_MODES[p])
        run.upload_initial()
        run.step(1)  # the first fused step creates the domain behind the arrays
    else:
        stream = torch.cuda.Stream()
        run = Runner(pkg, members, prec, ensemble, cap)
        run.set_stream(stream.cuda_stream)
        if ensemble and prec != abi.GBF_PREC_F64 and args.tile >= 0:
            run.set_tuning(args.tile, 0, 0)
            tuning = run.tuning()
        elif ensemble and prec != abi.GBF_PREC_F64 and not args.no_autotune:
            run.upload_initial()
            tuning = run.autotune(2)
        run.upload_initial()
    run.step(args.warmup)
    run.sync()
    cells, icells = W.cells, W.interior_cells
    with ClockSampler(torch.cuda.current_device()) as clk:
        ms = timed(run, args.steps, stream, world)            # value: graphs, no per-kernel events
        run.set_timing(True)                                   # roofline: the same steps with kernel events
        ms_k = timed(run, args.steps, stream, world)
    ktimes = run.kernel_times()
    run.set_timing(False)
    status = run.status()
    cells_job = dist_sum(float(cells), world)
    value = cells_job * args.steps / (ms / 1e3)

    # roofline of the dominant kernel
    hbm, peak_kind = peaks()
    kname, (kms, klaunch) = max(ktimes.items(), key=lambda kv: kv[1][0])
    per_launch_s = kms / 1e3 / max(klaunch, 1)
    table = ALGO_BYTES_DROPIN if p in DROPIN_MODES else ALGO_BYTES_DEFECT if p == "splitdefect" else ALGO_BYTES
    bpc, which = table.get(kname, ALGO_BYTES.get(kname, (0.0, "all")))
    algo = bpc * (icells if which == "interior" else cells)
    achieved = algo / per_launch_s / 1e9 if per_launch_s > 0 else 0.0
    traffic = None
    tfile = ROOT / "profiles" / "traffic.json"
    if tfile.exists():  # ncu DRAM bytes per cell of a smaller capture, scaled to this launch's cells
        ent = json.loads(tfile.read_text()).get(args.workload, {}).get(kname)
        if ent:
            traffic = ent["bytes_per_cell"] * (icells if ent["cells"] == "interior" else cells)
    f64 = "f64" in kname
    roof = {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm, "unit": "GB/s",
            "frac": achieved / hbm, "peak_source": peak_kind, "traffic": traffic,
            "algorithmic_bytes_per_launch": algo, "bytes_per_cell": bpc, "ms_per_launch": per_launch_s * 1e3,
            "kernel_times_ms": {k: {"total_ms": v[0], "launches": v[1]} for k, v in ktimes.items()},
            "binding_resource": ("FP64 pipe (ncu: 85% of FP64-pipe cycles active in the flux/Newton pass; "
                                 "GB300 DFMA 1.2 TFLOP/s)") if f64 else
                                ("instruction issue and the per-plane block barrier (ncu: 66-80% issue "
                                 "active; DRAM traffic 1.12-1.16x the algorithmic bytes on config 4, halo "
                                 "rows re-read)"),
            "ms_per_step_with_kernel_events": ms_k / args.steps}
    if f64:  # the FP64 kernels' own roof: the FP64 pipe, from the ncu capture of this pass
        roof["fp64_pipe"] = {"frac": 0.853, "metric": "sm__pipe_fp64_cycles_active",
                             "source": "profiles/f64_flux_newton_config1.md (flux/Newton pass, 192^3)"}

    # e2e through the public API with pinned host buffers: H2D state, one step, D2H P and S,
    # every step timed on its own (the host link is shared with other jobs on the host)
    e2e_steps = max(2, min(args.steps, 20))
    step_s = []
    if ensemble:
        Pall = torch.empty(cells, dtype=torch.float64, pin_memory=True).numpy()
        Sall = torch.empty(cells, dtype=torch.float64, pin_memory=True).numpy()
        run.download_all(Pall, Sall)
        for _ in range(max(1, args.warmup)):  # warm-up calls: the first sets up the pipeline's buffers
            run.advance_host(Pall, Sall, 1)
        torch.cuda.synchronize()
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            run.advance_host(Pall, Sall, 1)
            step_s.append(time.perf_counter() - t0)
        api = ("gbf_ensemble_advance_host(P, S, 1, P, S): every member's P1, S2 host->device, one step, "
               "device->host, pipelined over member groups")
    else:
        shape = members[0].model.shape
        hostP = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
        hostS = torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
        if p in DROPIN_MODES:
            def rt():
                run.upload(hostP, hostS)
                run.step(1)
                run.download("P1", hostP)
                run.download("S2", hostS)
            run.download("P1", hostP)
            run.download("S2", hostS)
            api = ("load_data_to_device(P1), load_data_to_device(S2), time_step_function's five calls, "
                   "load_data_to_host(P1), load_data_to_host(S2) (defines.h)")
        else:
            def rt():  # one call: upload, the step and the download pipelined over slabs of planes
                run.obj.advance_host(hostP, hostS, 1)
            run.download(0, "P1", hostP)
            run.download(0, "S2", hostS)
            api = ("gbf_domain_advance_host(P, S, 1, P, S): P1, S2 host->device, one step, device->host, "
                   "pipelined over slabs of planes (split forms without a Dirichlet patch; else the three calls)")
        for _ in range(max(1, args.warmup)):
            rt()
        torch.cuda.synchronize()
        for _ in range(e2e_steps):
            t0 = time.perf_counter()
            rt()
            step_s.append(time.perf_counter() - t0)
    # the median step is the typical cost; the mean, beside it, carries the
    # occasional slow step of the shared host (35-120 ms against 25 ms measured
    # for config 4, with the same copy rates)
    med_s = dist_max(statistics.median(step_s), world)
    mean_s = dist_max(sum(step_s) / len(step_s), world)
    link = link_bandwidth(torch)
    moved = 2 * cells * 8 * 2  # P, S each way, per step
    e2e = {"value": cells_job / med_s, "unit": "cell-steps/s", "statistic": f"median of {e2e_steps} timed steps",
           "mean_value": cells_job / mean_s, "step_ms": {"median": med_s * 1e3, "mean": mean_s * 1e3,
                                                        "min": min(step_s) * 1e3, "max": max(step_s) * 1e3},
           "h2d_bytes_per_step": 2 * cells * 8, "d2h_bytes_per_step": 2 * cells * 8, "api": api,
           "host_link": {"bytes_per_s": moved / med_s, "measured_pinned_copy_gbs": link,
                         "frac_of_concurrent_copy": moved / med_s / 1e9 / link["both_gbs"]}}

    out = {"metric": METRIC, "value": value, "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": PRECISIONS[p][2],
           "data": "synthetic (seeded fields with the configuration's shapes and statistics)",
           "config": W.config(),
           "details": {"dt_used_range": [min(m.model.dt for m in members), max(m.model.dt for m in members)],
                       "newton": ("converge-and-exit (tol 1e-11, at most the reference's 7)" if p == "dropin" else
                                  "increment Newton, a second iteration where nonlinear, one residual-correction "
                                  "step" if p == "dropinsplit" else
                                  "FP64: converge-and-exit (tol 1e-11, max 7); split: increment Newton, a second "
                                  "iteration where nonlinear, and (split) one residual-correction step"),
                       "tuning": tuning, "graphs": ensemble, "rank_cells": cells,
                       "plane_staging": ("none (FP64)" if p in ("f64", "dropin") else
                                         "TMA" if run.uses_tma else "plain loads")},
           "clocks": clk.summary(), "e2e": e2e,
           "gpu_launches": (run.launches_per_step if p not in DROPIN_MODES else run.lib.gbf_domain_launches_per_step(
               run.handle)) * args.steps,
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
            out["split_batched_over_fp64_batched"] = (cells * args.steps / (ms / 1e3)) / comp["f64"]["value"]
    if rank == 0 and not args.no_compare and p == "dropinsplit":
        out["accuracy"] = accuracy_dropin(pkg, members[0])
    elif rank == 0 and not args.no_compare and prec != abi.GBF_PREC_F64:
        O = ge.load_oracle_module()
        out["accuracy"] = accuracy_block(pkg, O, members, prec, ensemble)
        out["accuracy_stiff"] = accuracy_stiff(pkg, lib, W.wl, members, prec, ensemble)
    if rank == 0 and not args.no_cpu_baseline:
        O = ge.load_oracle_module()
        cb = reference_cpu_run(O, abi, members, steps=min(args.steps, 3), warmup=1, step_budget_s=step_budget(args))
        cb.pop("seconds", None)
        out["cpu_baseline"] = cb
    return out


def compare(pkg, members, prec, ensemble, steps, flags=0):
    """The same members advanced `steps` steps in form `prec` and in plain FP64
    on the GPU: both states and both phase-mass histories."""
    abi = pkg.abi

    def run(p):
        r = Runner(pkg, members, p, ensemble, steps + 2)
        if p != abi.GBF_PREC_F64:
            r.set_outputs(abi.GBF_OUT_MASS | flags, steps + 2)
        r.upload_initial()
        r.step(steps)
        out = [(r.download(i, "P1"), r.download(i, "S2")) for i in range(len(members))] if ensemble else \
            [(r.download(0, "P1"), r.download(0, "S2"))]
        mass = r.mass_history(steps)
        cfl = r.cfl_history(steps) if (flags & abi.GBF_OUT_CFL) and p != abi.GBF_PREC_F64 else None
        st = r.status()
        r.close()
        return out, mass, cfl, st

    got, mg, cfl, s1 = run(prec)
    ref, mr, _, s2 = run(abi.GBF_PREC_F64)
    ds = max(float(np.abs(a[1] - b[1]).max()) for a, b in zip(got, ref))
    num = sum(float(np.sum((a[0] - b[0]) ** 2)) for a, b in zip(got, ref))
    den = sum(float(np.sum(b[0] ** 2)) for b in ref)
    moved = max(float(np.abs(b[1] - m.initial_state()[1]).max()) for b, m in zip(ref, members))
    scale = np.maximum(np.abs(mr), 1e-300)
    drift = float(np.max(np.abs(mg - mr) / scale * (np.abs(mr) > 0)))
    block = {"vs": "plain FP64 GPU path of the same members (pinned to the oracle at 1e-12)", "steps": steps,
             "max_dS": ds, "rel_l2_P": (num / den) ** 0.5, "phase_mass_rel_diff_max": drift, "S_moved_max": moved,
             "status": [int(s1), int(s2)]}
    if cfl is not None:
        block["cfl_max"] = [float(cfl[..., 0].max()), float(cfl[..., 1].max())]
    return block, got


def accuracy_dropin(pkg, member, steps=20):
    """The drop-in's split mode against its fused FP64 mode (itself pinned to
    the oracle at 1e-12), both through the reference's calls from the same
    initial state for the same steps: max|dS|, relative L2 of P, and how far
    S moved (the DNAPL entering under the Dirichlet patch)."""
    out = {}
    for mode in (2, 1):
        run = DropinRunner(pkg, member, mode)
        run.upload_initial()
        run.step(steps)
        P = run.download("P1", np.empty(member.model.shape))
        S = run.download("S2", np.empty(member.model.shape))
        out[mode] = (P, S, int(run.status()))
        run.close()
    (Pg, Sg, s2), (Pr, Sr, s1) = out[2], out[1]
    S0 = member.initial_state()[1]
    return {"vs": "the drop-in's fused FP64 mode (pinned to the oracle at 1e-12), same calls and steps",
            "steps": steps, "max_dS": float(np.abs(Sg - Sr).max()),
            "rel_l2_P": float(np.linalg.norm(Pg - Pr) / np.linalg.norm(Pr)),
            "S_moved_max": float(np.abs(Sr - S0).max()), "status": [s2, s1]}


def accuracy_block(pkg, O, members, prec, ensemble, steps=20):
    """The measured form against plain FP64 on the same members and steps
    (the GPU FP64 path, itself pinned to the oracle at 1e-12), and against
    the oracle on the smallest member: max|dS|, relative L2 of P, relative
    phase-mass difference per step, and how far S moved (max|S - S0|)."""
    abi = pkg.abi
    block, got = compare(pkg, members, prec, ensemble, steps, abi.GBF_OUT_CFL)
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


def accuracy_stiff(pkg, lib, wl, members, prec, ensemble, steps=30, count=5):
    """The same comparison where the saturation moves: up to `count` members
    spanning the sizes, at the reference parameter file's compressibilities
    (1e-4 water, 1e-8 DNAPL) with 2 kg/s injected at half their stable dt."""
    import copy
    order = sorted(range(len(members)), key=lambda q: members[q].ncells)
    pick = sorted({order[round(k * (len(order) - 1) / max(1, count - 1))] for k in range(min(count, len(order)))})
    sel = []
    for q in pick:
        m = copy.copy(members[q])
        m.model = members[q].model.copy()
        m.model.beta1, m.model.beta2 = 1e-4, 1e-8
        if m.model.source_mode == pkg.abi.GBF_SOURCE_RATE:
            m.model.rate = 2.0
        m.model.newton_tol = 1e-11
        sel.append(wl.set_stable_dt(lib, m, 0.5))
    block, _ = compare(pkg, sel, prec, ensemble, steps)
    block["members"] = pick
    block["params"] = "beta1 1e-4, beta2 1e-8, 2 kg/s, dt = 0.5 x stable"
    return block


# ------------------------------------------------------------- reference arm

def run_reference(args, rank, world):
    """The reference CPU algorithm (oracle) on all host cores, same workload,
    metric and config; inputs from libgbf_inputs.so (libgbflow not loaded)."""
    if rank != 0:
        return None
    pkg = ge.load_package()
    O = ge.load_oracle_module()
    lib = O.inputs_library(pkg.abi)
    W = Workload(pkg, lib, args.workload, args.cube, 0, world, args.members)
    cb = reference_cpu_run(O, pkg.abi, W.members, args.steps, args.warmup, step_budget(args))
    v = cb["value"]
    return {"metric": METRIC, "impl": "reference", "value": v, "unit": "cell-steps/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * cb.pop("seconds") / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded fields with the configuration's shapes and statistics)",
            "config": W.config(),
            "details": {"arm": "reference CPU algorithm in FP64 (the bit-exact port of cpu.cpp) on rank 0's "
                               "members; inputs from libgbf_inputs.so"},
            "e2e": {"value": v, "unit": "cell-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cpu_baseline": cb}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="config4_split")
    ap.add_argument("--cube", type=int, default=0, help="override the grid edge of config1 (profiling runs)")
    ap.add_argument("--members", type=int, default=0, help="first N members of an ensemble (profiling runs)")
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
