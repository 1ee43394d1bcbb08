"""Parity with the oracle (the reference's CPU algorithm) at the benchmark
configurations' own sizes, and the split forms over the configurations' own
step counts.

- config 1, 256^3 with its heterogeneous fields: plain FP64 through the
  domain API; and config 1's grid through the reference's own host function
  set (defines.h, fused mode) in the media-table physics those calls express;
  3 steps each against the oracle (7 Newton iterations there, converge-and-
  exit on the GPU): max|dS| <= 1e-12, P within the FP64 tolerance, phase
  masses within 1e-12 every step.
- config 2, 512x512x256: the split form (masses at FP64 precision, residual
  correction) and the FP32-defect form, 2 steps against the oracle: max|dS|
  <= 1e-5, relative L2 of P <= 1e-6, phase masses within 1e-9 every step.
- config 4: the whole 256-member ensemble in the split form and in plain
  FP64 on the GPU, five members spanning the edge range against the oracle,
  3 steps, with the same gates.
All at the configurations' own compressibility (1e-9), where the saturation
barely moves in a few steps (the pressure carries the comparison there; the
long runs below and the split tests move the saturation).

The long runs: config 4 for 1000 steps and config 3 for 500 steps, the split
form against plain FP64 on the GPU at the reference parameter file's
compressibilities (1e-4 water, 1e-8 DNAPL; half their stable dt), each
member's phase masses within 1e-9 every step and max|dS| <= 1e-5 at the end.
Each test prints the numbers it measured.
"""
from importlib import import_module

import numpy as np
import pytest

from gpu_util import F64_TOL, p_tol, rel_l2

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def wl(pkg):
    return import_module(pkg.__name__ + ".workloads")


def oracle_run(O, oracle, mem, steps):
    """The oracle from the member's initial state: final state, masses per step."""
    m = mem.model.copy()
    m.newton_tol = 0.0  # the reference's 7 iterations
    st = O.State(m, mem.media, mem.K, mem.phi)
    P, S = mem.initial_state()
    st["P1"][...] = P
    st["S2"][...] = S
    mass = oracle.step(st, steps, want_mass=True)
    return st, mass


def mass_rel(got, want):
    scale = np.where(np.abs(want) > 0, np.abs(want), 1.0)
    return float(np.max(np.abs(got - want) / scale))


def check_f64(name, P, S, mass, st, ref_mass, m):
    ds = float(np.abs(S - st["S2"]).max())
    pmax = float(np.abs(P - st["P1"]).max() / np.abs(st["P1"]).max())
    pl2 = rel_l2(P, st["P1"])
    mr = mass_rel(mass, ref_mass) if mass is not None else None
    print(f"\n{name}: max|dS| {ds:.2e}, max|dP|/max|P| {pmax:.2e}, rel-L2(P) {pl2:.2e}, mass {mr}")
    assert ds <= F64_TOL
    assert pmax <= p_tol(m) and pl2 <= p_tol(m)
    if mr is not None:
        assert mr <= 1e-12


def test_config1_fp64_domain_matches_oracle_at_256_cubed(gpu_lib, abi, O, oracle, pkg, wl):
    Domain = import_module(pkg.__name__ + ".domain").Domain
    mem = wl.config1(gpu_lib)
    assert mem.model.shape == (256, 256, 256) and mem.model.newton_tol > 0
    steps = 3
    st, ref_mass = oracle_run(O, oracle, mem, steps)
    d = Domain(mem.model, mem.media, mem.K, mem.phi, precision=abi.GBF_PREC_F64)
    d.set_outputs(abi.GBF_OUT_MASS, steps)
    d.upload(*mem.initial_state())
    d.step(steps)
    assert d.status() == abi.GBF_OK
    check_f64("config 1 FP64 domain", d.download("P1"), d.download("S2"), d.mass_history(steps), st, ref_mass,
              mem.model)
    d.close()


def test_config1_dropin_fused_matches_oracle_at_256_cubed(gpu_lib, abi, O, oracle, pkg, wl):
    """time_step_function's five defines.h calls per step (main.cpp:83-94),
    fused mode, on config 1's 256^3 grid."""
    import ctypes
    dp = import_module(pkg.__name__ + ".dropin")
    mem = wl.config1_dropin(gpu_lib)
    m = mem.model
    steps = 3
    st, _ = oracle_run(O, oracle, mem, steps)
    di = dp.DropIn()
    di.set_mode(1)
    c = dp.consts_from_model(m)
    H, D = dp.PtrArrays(), dp.PtrArrays()
    buf = ctypes.c_void_p()
    di.f["device_memory_alloc"](ctypes.byref(D), ctypes.byref(buf), m.nx, c)
    assert gpu_lib.gbf_last_status() == 0
    P0, S0 = mem.initial_state()
    di.f["load_data_to_device"](P0.ctypes.data, D.P1, m.nx, c)
    di.f["load_data_to_device"](S0.ctypes.data, D.S2, m.nx, c)
    di.f["load_data_to_device_int"](np.ascontiguousarray(mem.media).ctypes.data, D.media, m.nx, c)
    for s in range(1, steps + 1):
        di.time_step(H, D, c, s * m.dt)
    out = {}
    for name in ("P1", "S2"):
        out[name] = np.empty(m.shape, np.float64)
        di.f["load_data_to_host"](out[name].ctypes.data, getattr(D, name), m.nx, c)
    assert gpu_lib.gbf_last_status() == 0
    di.f["device_memory_free"](D, buf)
    di.set_mode(0)
    check_f64("config 1 drop-in (fused)", out["P1"], out["S2"], None, st, None, m)


@pytest.mark.parametrize("form", ["split", "split_defect"])
def test_config2_split_forms_match_oracle_at_full_size(gpu_lib, abi, O, oracle, pkg, wl, form):
    Domain = import_module(pkg.__name__ + ".domain").Domain
    prec = {"split": abi.GBF_PREC_SPLIT, "split_defect": abi.GBF_PREC_SPLIT_DEFECT}[form]
    mem = wl.config2(gpu_lib)
    assert mem.model.shape == (256, 512, 512)
    steps = 2
    st, ref_mass = oracle_run(O, oracle, mem, steps)
    d = Domain(mem.model, mem.media, mem.K, mem.phi, precision=prec)
    d.set_outputs(abi.GBF_OUT_MASS, steps)
    d.upload(*mem.initial_state())
    d.step(steps)
    assert d.status() == abi.GBF_OK
    P, S, mass = d.download("P1"), d.download("S2"), d.mass_history(steps)
    d.close()
    ds, pl2, mr = float(np.abs(S - st["S2"]).max()), rel_l2(P, st["P1"]), mass_rel(mass, ref_mass)
    print(f"\nconfig 2 {form}: max|dS| {ds:.2e}, rel-L2(P) {pl2:.2e}, mass {mr:.2e}")
    assert ds <= 1e-5 and pl2 <= 1e-6 and mr <= 1e-9


def test_config4_members_match_oracle(gpu_lib, abi, O, oracle, pkg, wl):
    """The whole ensemble on the GPU (split form and plain FP64); five members
    spanning the edges against the oracle."""
    E = import_module(pkg.__name__ + ".ensemble").Ensemble
    members = wl.config4(gpu_lib)
    assert len(members) == 256
    steps = 3
    order = sorted(range(len(members)), key=lambda r: (members[r].model.nx, r))
    pick = [order[round(q * (len(order) - 1) / 4)] for q in range(5)]
    assert len({members[r].model.nx for r in pick}) >= 4
    refs = {r: oracle_run(O, oracle, members[r], steps) for r in pick}
    for prec, name in ((abi.GBF_PREC_SPLIT, "split"), (abi.GBF_PREC_F64, "f64")):
        e = E(members, precision=prec)
        e.set_outputs(abi.GBF_OUT_MASS, steps)
        e.upload_initial()
        e.step(steps)
        e.sync()
        assert e.status() == abi.GBF_OK
        mass = e.mass_history(steps)
        for r in pick:
            st, ref_mass = refs[r]
            P, S = e.download(r, "P1"), e.download(r, "S2")
            if name == "f64":
                check_f64(f"config 4 member {r} ({members[r].model.nx}^3) FP64", P, S, mass[:, r], st, ref_mass,
                          members[r].model)
            else:
                ds, pl2, mr = float(np.abs(S - st["S2"]).max()), rel_l2(P, st["P1"]), mass_rel(mass[:, r], ref_mass)
                print(f"\nconfig 4 member {r} ({members[r].model.nx}^3) split: max|dS| {ds:.2e}, "
                      f"rel-L2(P) {pl2:.2e}, mass {mr:.2e}")
                assert ds <= 1e-5 and pl2 <= 1e-6 and mr <= 1e-9
        e.close()


def stiff(wl, lib, members):
    for mem in members:
        mem.model.beta1, mem.model.beta2 = 1e-4, 1e-8
        mem.model.newton_tol = 1e-11
        wl.set_stable_dt(lib, mem, 0.5)
    return members


@pytest.mark.parametrize("cfg,steps", [("config4", 1000), ("config3", 500)])
def test_split_over_the_configurations_step_counts(gpu_lib, abi, pkg, wl, cfg, steps):
    E = import_module(pkg.__name__ + ".ensemble").Ensemble
    members = stiff(wl, gpu_lib, getattr(wl, cfg)(gpu_lib))
    out = {}
    for prec, name in ((abi.GBF_PREC_F64, "f64"), (abi.GBF_PREC_SPLIT, "split")):
        e = E(members, precision=prec)
        e.set_outputs(abi.GBF_OUT_MASS, steps)
        e.upload_initial()
        e.step(steps)
        e.sync()
        assert e.status() == abi.GBF_OK, name
        out[name] = (e.mass_history(steps), [(e.download(r, "P1"), e.download(r, "S2")) for r in range(len(members))])
        e.close()
    mr, ref = out["f64"]
    md, got = out["split"]
    assert md.shape == mr.shape == (steps, len(members), 2)
    drift = mass_rel(md, mr)
    ds = max(float(np.abs(b[1] - a[1]).max()) for a, b in zip(ref, got))
    num = sum(float(np.sum((b[0] - a[0]) ** 2)) for a, b in zip(ref, got))
    den = sum(float(np.sum(a[0] ** 2)) for a in ref)
    moved = max(float(np.abs(a[1] - m.initial_state()[1]).max()) for a, m in zip(ref, members))
    print(f"\n{cfg} {steps} steps, split vs FP64: max|dS| {ds:.2e}, rel-L2(P) {(num / den) ** 0.5:.2e}, "
          f"mass drift (every member and step) {drift:.2e}, S moved {moved:.2e}")
    assert moved > 1e-3
    assert ds <= 1e-5 and (num / den) ** 0.5 <= 1e-6 and drift <= 1e-9
