"""Run the reference's own driver (main.cpp + no_communication.cpp, unmodified)
against libgbflow.so on the GPU and against the reference CPU backend
(cpu.cpp), and compare every output file.

    python tests/reference_driver/run_reference_driver.py <reference-dir> <out-dir>

<reference-dir> holds the reference sources (main.cpp, no_communication.cpp,
cpu.cpp, defines.h); they are compiled where they lie, nothing is copied or
edited. Two binaries are linked the way the reference's build scripts link
them (sh/cpu.sh, sh/cuda.sh): filtration_cpu with cpu.cpp, filtration_gb300
with libgbflow.so in place of gpu.cu.

defines.h fixes the parameter file's path to the Windows path
"C://Users//.../Buckley-Leverett//defines.ini"; on Linux that is a relative
path, so every run gets a working directory holding a parameter file at
exactly that path. The file sets a 15^3 grid with the reference's physics and
dt = 0.02 s (below the explicit bound of 0.040 s): the driver's loop runs
timeX / dt = 25000 steps and writes its Tecplot files every 5000 steps.

Scenarios, each run by the CPU build and the GB300 build in eager mode, in
fused mode (GBF_DROPIN_MODE=1) and in split mode (GBF_DROPIN_MODE=2, the
headline split form behind the same calls):
  fresh    initial_data (main.cpp:97-138), steps 1..25000;
  restart  save/save.dat present, written by gbf_checkpoint_write from the
           oracle's state after 12500 steps: restore (main.cpp:541-572), then
           steps 12501..25000.
Every file the CPU build writes (plot_*/*.dat, media.dat) must exist in the
GB300 runs. The eager mode, which runs the reference's arithmetic, must write
them byte for byte; the fused mode (log/exp instead of pow, FMA, a
converge-and-exit Newton) values within FUSED_TOL of each column's largest
magnitude, beyond last printed digits that flip where a value sits on a
rounding boundary; the split mode within SPLIT_TOL of each column's largest
magnitude over the plot kind's files. Prints one JSON summary line; exit code 0 when all match.
"""
from __future__ import annotations

import ctypes
import json
import os
import pathlib
import subprocess
import sys
import time

ROOT = pathlib.Path(__file__).resolve().parents[2]
LIBDIR = ROOT / "shmem-cuda-filtration_gb300" / "_build"
INI_DIR = pathlib.Path("C:", "Users", "dmitry", "Documents", "Visual Studio 2010", "Projects", "Buckley-Leverett")
STEPS, DT, SAVE_EVERY = 25000, 0.02, 5000
# Fused mode against the CPU build: P and S agree with the oracle to 1e-12
# and the velocities, first differences of P over h, to 1e-10 of their
# largest magnitude after a few steps (the drop-in tests); here after 25000
# steps, where near-hydrostatic columns carry velocities many orders below
# the largest, the bar is on each column's largest magnitude.
FUSED_TOL = 1e-8
# Split mode: FP32 state and fluxes with FP64-precision masses. On the 15^3
# grid the printed columns (P1, S2, the velocities) measured at most 1.7e-8 of
# their scale, the largest magnitude a column takes over its plot kind's time
# series (5e-15 after the restart); the bar keeps a factor of about 60. A
# column's own maximum in one early file is no scale: S2 far from the DNAPL
# holds round-off of 1e-17 there, and 4e-19 moves it by 1e-2 of that.
SPLIT_TOL = 1e-6
NX = NY = NZ = 15

# The reference parameter file's keys (main.cpp:601-684) with its values,
# except DT, SAVE_PLOTS and PRINT_SCREEN.
PARAMS = [("H1", "0.02045"), ("H2", "0.01969"), ("H3", "0.01969"), ("DT", str(DT)), ("TAU", "0.002"),
          ("L_N", "8.528784e-10"), ("L_W", "2e-7"), ("C", "1407"), ("BETA1", "1.0e-4"), ("BETA2", "1.0e-8"),
          ("NX", str(NX)), ("NY", str(NY)), ("NZ", str(NZ)), ("SOURCE", "3"), ("SAVE_PLOTS", str(SAVE_EVERY)),
          ("PRINT_SCREEN", str(SAVE_EVERY)), ("K[0]", "6.64e-11"), ("K[1]", "7.15e-12"), ("MU1", "0.001"),
          ("MU2", "0.0009"), ("RO_W", "1000"), ("RO_N", "1460"), ("LAMBDA[0]", "2.7"), ("LAMBDA[1]", "2.0"),
          ("S_WR[0]", "0.09"), ("S_WR[1]", "0.12"), ("S2_GR", "0.4"), ("M[0]", "0.4"), ("M[1]", "0.39"),
          ("P_D[0]", "755"), ("P_D[1]", "2060"), ("P_ATM", "100000"), ("G_CONST", "9.8")]


def build(ref: pathlib.Path, out: pathlib.Path) -> dict:
    out.mkdir(parents=True, exist_ok=True)
    common = ["g++", "-O2", "-ffp-contract=off", "-w", f"-I{ref}", str(ref / "main.cpp"),
              str(ref / "no_communication.cpp")]
    cmds = {"cpu": common + [str(ref / "cpu.cpp"), "-o", str(out / "filtration_cpu")],
            "gb300": common + [f"-L{LIBDIR}", "-lgbflow", f"-Wl,-rpath,{LIBDIR}", "-o", str(out / "filtration_gb300")]}
    for name, cmd in cmds.items():
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise SystemExit(f"build of {name} failed:\n{r.stderr[-3000:]}")
    return {"cpu": out / "filtration_cpu", "gb300": out / "filtration_gb300"}


def write_checkpoint(path: pathlib.Path, steps: int) -> None:
    """save/save.dat of the oracle's state after `steps` steps, in the
    reference's checkpoint layout (gbf_checkpoint_write)."""
    sys.path.insert(0, str(ROOT))
    import __graft_entry__ as ge
    pkg = ge.load_package()
    abi, lib = pkg.abi, pkg.load_library()
    O = ge.load_oracle_module()
    m = abi.reference_model(NX, NY, NZ, DT)
    st = O.State(m)
    orc = O.Oracle(abi)
    orc.initial(st)
    orc.step(st, steps)
    lib.gbf_checkpoint_write.restype = ctypes.c_int
    path.parent.mkdir(parents=True, exist_ok=True)
    d = lambda a: a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))  # noqa: E731
    rc = lib.gbf_checkpoint_write(str(path).encode(), ctypes.byref(m), steps, d(st["P1"]), d(st["S2"]),
                                  d(st["roS1_old"]), d(st["roS2_old"]),
                                  st.media.ctypes.data_as(ctypes.POINTER(ctypes.c_int)))
    if rc != 0:
        raise SystemExit(f"gbf_checkpoint_write: {rc}")


def run(exe: pathlib.Path, wd: pathlib.Path, env_mode: str | None, checkpoint: pathlib.Path | None) -> dict:
    wd.mkdir(parents=True, exist_ok=True)
    (wd / INI_DIR).mkdir(parents=True, exist_ok=True)
    (wd / INI_DIR / "defines.ini").write_text("".join(f"{k}={v}\n" for k, v in PARAMS))
    if checkpoint is not None:
        (wd / "save").mkdir(exist_ok=True)
        (wd / "save" / "save.dat").write_bytes(checkpoint.read_bytes())
    env = dict(os.environ)
    env.pop("GBF_DROPIN_MODE", None)
    if env_mode is not None:
        env["GBF_DROPIN_MODE"] = env_mode
    t0 = time.perf_counter()
    r = subprocess.run([str(exe)], cwd=wd, env=env, capture_output=True, text=True, stdin=subprocess.DEVNULL)
    dt = time.perf_counter() - t0
    (wd / "stdout.txt").write_text(r.stdout + r.stderr)
    return {"rc": r.returncode, "seconds": dt, "task_time": next((ln.split()[-1] for ln in r.stdout.splitlines()
                                                                  if ln.startswith("Task time")), None)}


def outputs(wd: pathlib.Path) -> list[str]:
    files = [p.relative_to(wd).as_posix() for p in wd.rglob("*.dat") if p.parent.name.startswith("plot_")]
    return sorted(files + (["media.dat"] if (wd / "media.dat").exists() else []))


def _unit(tok: str) -> float:
    """One unit of the last printed digit of a number printed as %.Ne or %d."""
    s = tok.lower()
    mant, _, exp = s.partition("e")
    digits = len(mant.split(".")[1]) if "." in mant else 0
    return 10.0 ** ((int(exp) if exp else 0) - digits)


def column_scales(files) -> dict:
    """Largest magnitude of each numeric column over a set of files (one plot
    kind's time series)."""
    out = {}
    for f in files:
        for ln in f.read_text().splitlines():
            for c, u in enumerate(ln.split()):
                try:
                    out[c] = max(out.get(c, 0.0), abs(float(u)))
                except ValueError:
                    pass
    return out


def compare(a: pathlib.Path, b: pathlib.Path, scales: dict | None = None) -> dict:
    """Byte equality; else, value by value, the differences beyond one unit of
    the last printed digit (a value on a rounding boundary may print either
    way) relative to the column's scale: the largest magnitude of the column in
    this file or, when larger, over the plot kind's whole time series
    (`scales`; a column that holds round-off far from the DNAPL at one time,
    1e-17, is measured on the values it takes later)."""
    ba, bb = a.read_bytes(), b.read_bytes()
    if ba == bb:
        return {"equal": True}
    la, lb = ba.decode().splitlines(), bb.decode().splitlines()
    if len(la) != len(lb):
        return {"equal": False, "lines": [len(la), len(lb)], "max_rel": float("inf")}
    rows = [(x.split(), y.split()) for x, y in zip(la, lb)]
    colmax = dict(scales or {})
    for x, _ in rows:
        for c, u in enumerate(x):
            try:
                colmax[c] = max(colmax.get(c, 0.0), abs(float(u)))
            except ValueError:
                pass
    flips, beyond, worst = 0, 0, {}
    for x, y in rows:
        if x == y:
            continue
        if len(x) != len(y):
            return {"equal": False, "text": [" ".join(x), " ".join(y)], "max_rel": float("inf")}
        for c, (u, v) in enumerate(zip(x, y)):
            if u == v:
                continue
            try:
                fu, fv = float(u), float(v)
            except ValueError:
                return {"equal": False, "text": [" ".join(x), " ".join(y)], "max_rel": float("inf")}
            d = abs(fu - fv)
            if d <= max(_unit(u), _unit(v)) * (1 + 1e-9):
                flips += 1
                continue
            beyond += 1
            worst[c] = max(worst.get(c, 0.0), d / colmax[c] if colmax.get(c) else float("inf"))
    return {"equal": False, "last_digit_flips": flips, "beyond_one_digit": beyond,
            "max_rel_by_column": {str(c): w for c, w in sorted(worst.items())},
            "max_rel": max(worst.values(), default=0.0)}


def main():
    ref, out = pathlib.Path(sys.argv[1]).resolve(), pathlib.Path(sys.argv[2]).resolve()
    for f in ("main.cpp", "no_communication.cpp", "cpu.cpp", "defines.h"):
        if not (ref / f).exists():
            raise SystemExit(f"{ref / f} missing")
    exes = build(ref, out / "bin")
    ckpt = out / "checkpoint_12500.dat"
    write_checkpoint(ckpt, STEPS // 2)
    summary = {"steps": STEPS, "dt": DT, "grid": [NX, NY, NZ], "scenarios": {}}
    ok = True
    for scen, cp in (("fresh", None), ("restart", ckpt)):
        runs = {"cpu": run(exes["cpu"], out / scen / "cpu", None, cp),
                "gb300_eager": run(exes["gb300"], out / scen / "gb300_eager", "0", cp),
                "gb300_fused": run(exes["gb300"], out / scen / "gb300_fused", "1", cp),
                "gb300_split": run(exes["gb300"], out / scen / "gb300_split", "2", cp)}
        files = outputs(out / scen / "cpu")
        res = {"runs": runs, "files": len(files), "compare": {}}
        ok &= all(r["rc"] == 0 for r in runs.values()) and len(files) > 0
        for mode in ("gb300_eager", "gb300_fused", "gb300_split"):
            got = outputs(out / scen / mode)
            c = {"missing": sorted(set(files) - set(got)), "extra": sorted(set(got) - set(files))}
            kinds = {pathlib.PurePosixPath(f).parent for f in files}
            scales = {k: column_scales([out / scen / "cpu" / f for f in files if pathlib.PurePosixPath(f).parent == k])
                      for k in kinds}
            per = {f: compare(out / scen / "cpu" / f, out / scen / mode / f, scales[pathlib.PurePosixPath(f).parent])
                   for f in files if f in got}
            c["byte_equal"] = sum(1 for v in per.values() if v["equal"])
            c["differing"] = {f: v for f, v in per.items() if not v["equal"]}
            # eager mode runs the reference's own arithmetic: byte equality;
            # fused mode (log/exp, FMA, converge-and-exit Newton): values
            # within FUSED_TOL of their column's scale beyond digit flips
            tol = {"gb300_eager": 0.0, "gb300_fused": FUSED_TOL, "gb300_split": SPLIT_TOL}[mode]
            c["max_rel"] = max((v["max_rel"] for v in c["differing"].values()), default=0.0)
            ok &= not c["missing"] and c["max_rel"] <= tol and (mode != "gb300_eager" or not c["differing"])
            res["compare"][mode] = c
        summary["scenarios"][scen] = res
    summary["ok"] = bool(ok)
    print(json.dumps(summary))
    sys.exit(0 if ok else 1)


if __name__ == "__main__":
    main()
