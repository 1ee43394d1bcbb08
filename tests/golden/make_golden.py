"""Generate the golden fixtures from the reference's own CPU backend.

The reference (cpu.cpp + main.cpp + no_communication.cpp) has no tests and no
golden vectors, so these fixtures are made by running it: oracle/Makefile
compiles those files from their sources into oracle/_ref/libgbf_refcpu.so and
this script drives them through their own functions (initial_data,
time_step_function, the five hot-path calls, the checkpoint writer save and
the Tecplot writer save_data_plots).

Run from the repository root, with GBF_REFERENCE_DIR naming the reference
checkout (oracle/Makefile compiles it from there):
    GBF_REFERENCE_DIR=<reference checkout> python tests/golden/make_golden.py
Outputs tests/golden/*.npz (small, committed).
"""
from __future__ import annotations

import json
import pathlib
import sys
import tempfile

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))
import __graft_entry__ as ge  # noqa: E402

OUT = pathlib.Path(__file__).resolve().parent
SAVED = ["P1", "S2", "roS1", "roS2", "u2x", "u2y", "u2z"]


def model_dict(m):
    return {f[0]: (list(getattr(m, f[0])) if f[0] in ("K", "lam", "S_wr", "m", "P_d") else getattr(m, f[0]))
            for f in m._fields_}


def random_state(O, m, seed):
    """A perturbed, non-equilibrium state: hydrostatic P plus noise, random S2."""
    rng = np.random.default_rng(seed)
    media = (rng.random(m.shape) < 0.35).astype(np.int32)
    st = O.State(m, media)
    j = np.arange(m.ny, dtype=np.float64)[None, :, None]
    st["P1"][...] = m.P_atm + j * m.ro01 * m.g * m.h2 + rng.uniform(-40.0, 40.0, m.shape)
    st["S2"][...] = rng.uniform(0.0, 0.45, m.shape)
    return st


def main():
    abi = ge.load_package().abi
    O = ge.load_oracle_module()
    O.build()
    if not O.Reference.available():
        raise SystemExit("reference library not built (reference sources absent)")
    ref = O.Reference()

    # 1-2: multi-step runs from the reference's own initial_data.
    runs = [
        ("ref_run_15cube_dt0.02_100steps", (15, 15, 15), 0.02, 100, 3, False),
        ("ref_run_13x17x19_media_dt0.02_60steps", (13, 17, 19), 0.02, 60, 2, True),
    ]
    for name, (nx, ny, nz), dt, steps, source, mixed in runs:
        m = abi.reference_model(nx, ny, nz, dt)
        m.source = source
        media = None
        if mixed:
            media = (np.random.default_rng(7).random(m.shape) < 0.3).astype(np.int32)
        st = O.State(m, media)
        ref.initial(st)
        ref.step(st, steps)
        np.savez_compressed(OUT / f"{name}.npz", model=json.dumps(model_dict(m)), steps=steps,
                            media=st.media.astype(np.int8), **{k: st[k] for k in SAVED})
        print(name, "S2 max", st["S2"].max())

    # 3: one call of each hot-path function in time_step_function's order on a
    # random state; every stage's outputs are stored.
    m = abi.reference_model(8, 9, 10, 0.02)
    m.source = 1
    st = random_state(O, m, 11)
    stages = {"in_P1": st["P1"].copy(), "in_S2": st["S2"].copy(), "media": st.media.astype(np.int8)}
    ref.props(st)
    for k in ("P2", "Xi1", "Xi2", "ro1", "ro2"):
        stages[f"props_{k}"] = st[k].copy()
    ref.velocity(st)
    for k in ("u1x", "u1y", "u1z", "u2x", "u2y", "u2z"):
        stages[f"velocity_{k}"] = st[k].copy()
    ref.mass(st, t=1.0)
    for k in ("roS1", "roS2", "roS1_old", "roS2_old"):
        stages[f"mass_{k}"] = st[k].copy()
    ref.newton(st)
    for k in ("P1", "S2"):
        stages[f"newton_{k}"] = st[k].copy()
    ref.boundary(st)
    for k in ("P1", "S2"):
        stages[f"boundary_{k}"] = st[k].copy()
    np.savez_compressed(OUT / "ref_stages_8x9x10.npz", model=json.dumps(model_dict(m)), **stages)

    # 4: a checkpoint file written by the reference's own save() (main.cpp:485)
    # after 7 steps of a run from initial_data; the file's bytes are stored.
    m = abi.reference_model(10, 8, 6, 0.02)
    m.source = 1
    st = O.State(m)
    ref.initial(st)  # sets media to 0; mixed media afterwards
    st.media[...] = (np.random.default_rng(5).random(m.shape) < 0.3).astype(np.int32)
    ref.step(st, 7)
    with tempfile.TemporaryDirectory() as d:
        ref.save(st, d, 7)
        dat = (pathlib.Path(d) / "save" / "save.dat").read_bytes()
    np.savez_compressed(OUT / "ref_checkpoint_10x8x6_step7.npz", model=json.dumps(model_dict(m)), steps=7,
                        dat=np.frombuffer(dat, np.uint8))
    # 5: the Tecplot files of the reference's save_data_plots() (main.cpp:319)
    # after 4 steps (odd Ny: the S2_x profile's row offset is nx*ny/2).
    m = abi.reference_model(9, 7, 5, 0.02)
    m.source = 1
    st = O.State(m)
    ref.initial(st)
    st.media[...] = (np.random.default_rng(6).random(m.shape) < 0.3).astype(np.int32)
    ref.step(st, 4)
    t = 4 * m.dt
    files = {}
    with tempfile.TemporaryDirectory() as d:
        ref.plots(st, d, t)
        for f in sorted(pathlib.Path(d).rglob("*.dat")):
            files["file:" + str(f.relative_to(d))] = np.frombuffer(f.read_bytes(), np.uint8)
    np.savez_compressed(OUT / "ref_plots_9x7x5_step4.npz", model=json.dumps(model_dict(m)), t=t,
                        media=st.media.astype(np.int8), **{k: st[k] for k in ("P1", "S2", "u2x", "u2y", "u2z")},
                        **files)
    for p in sorted(OUT.glob("*.npz")):
        print(p.name, p.stat().st_size)


if __name__ == "__main__":
    main()
