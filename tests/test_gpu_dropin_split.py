"""The drop-in's split mode (gbf_dropin_set_mode(2), GBF_DROPIN_MODE=2): the
reference's defines.h calls, time_step_function's five per step, run the
headline split form (FP32 state and fluxes, FP64-precision masses, one
residual-correction Newton step per cell) beside the caller's FP64 arrays.
Against the oracle (the reference's cpu.cpp arithmetic) on a reference grid
with its Dirichlet patch and the reference parameter file's physics, at the
split form's bars: max|dS| <= 1e-5, rel-L2(P) <= 1e-6; the derived arrays
the host reads (P2, ro1, ro2, from the state the last step started from)
as well. Also: P1 and S2 written by the host in the middle of a run (the
split state is formed anew from them), and a change to the eager mode in the
middle of a run (the caller's arrays are brought up to date first), and a
media array rewritten by the host after the split domain exists (its mass
sums then use the new porosities).
"""
import ctypes
from importlib import import_module

import numpy as np
import pytest

from gpu_util import rel_l2

pytestmark = pytest.mark.gpu

SHAPE = (48, 40, 44)
DT = 0.02
DS_TOL, P_TOL = 1e-5, 1e-6


@pytest.fixture
def dropin(pkg, gpu_lib):
    dp = import_module(pkg.__name__ + ".dropin")
    di = dp.DropIn()
    yield dp, di
    di.set_mode(0)


def oracle_states(abi, O, steps):
    """The oracle from initial_data: the state after each of `steps` (dict of copies)."""
    m = abi.reference_model(*SHAPE, DT)
    st = O.State(m)
    orc = O.Oracle(abi)
    orc.initial(st)
    out = {0: st.copy()}
    for s in steps:
        orc.step(st, s - max(out))
        out[s] = st.copy()
    return m, out


class Run:
    """Arrays from device_memory_alloc, the oracle's initial state loaded."""

    def __init__(self, dp, di, m, st0):
        self.dp, self.di, self.m = dp, di, m
        self.c = dp.consts_from_model(m)
        self.H, self.D = dp.PtrArrays(), dp.PtrArrays()
        self.buf = ctypes.c_void_p()
        di.f["device_memory_alloc"](ctypes.byref(self.D), ctypes.byref(self.buf), m.nx, self.c)
        self.put("P1", st0["P1"])
        self.put("S2", st0["S2"])
        self.t = 0

    def put(self, name, a):
        a = np.ascontiguousarray(a, np.float64)
        self.di.f["load_data_to_device"](a.ctypes.data, getattr(self.D, name), self.m.nx, self.c)

    def put_media(self, media):
        a = np.ascontiguousarray(media, np.int32)
        self.di.f["load_data_to_device_int"](a.ctypes.data, self.D.media, self.m.nx, self.c)

    def get(self, name):
        out = np.empty(self.m.shape, np.float64)
        self.di.f["load_data_to_host"](out.ctypes.data, getattr(self.D, name), self.m.nx, self.c)
        return out

    def steps(self, n):
        for _ in range(n):
            self.t += 1
            self.di.time_step(self.H, self.D, self.c, self.t * self.m.dt)

    def close(self):
        self.di.f["device_memory_free"](self.D, self.buf)


def check(tag, run, st, derived=False):
    P, S = run.get("P1"), run.get("S2")
    ds, pl2 = float(np.abs(S - st["S2"]).max()), rel_l2(P, st["P1"])
    line = f"{tag}: max|dS| {ds:.2e}, rel-L2(P) {pl2:.2e}"
    assert ds <= DS_TOL and pl2 <= P_TOL, line
    if derived:
        P2, r1, r2 = rel_l2(run.get("P2"), st["P2"]), rel_l2(run.get("ro1"), st["ro1"]), rel_l2(run.get("ro2"), st["ro2"])
        line += f", P2 {P2:.2e}, ro1 {r1:.2e}, ro2 {r2:.2e}"
        assert P2 <= P_TOL and r1 <= P_TOL and r2 <= P_TOL, line
    print("\n" + line)


def test_split_mode_matches_oracle(gpu_lib, abi, O, dropin):
    dp, di = dropin
    m, st = oracle_states(abi, O, [20])
    assert np.abs(st[20]["S2"] - st[0]["S2"]).max() > 1e-3  # DNAPL enters through the patch
    di.set_mode(2)
    run = Run(dp, di, m, st[0])
    run.steps(20)
    assert gpu_lib.gbf_last_status() == abi.GBF_OK
    check("split mode, 20 steps", run, st[20], derived=True)
    run.close()


def test_split_mode_host_writes_and_mode_change(gpu_lib, abi, O, dropin):
    dp, di = dropin
    m, st = oracle_states(abi, O, [10, 20, 30])
    di.set_mode(2)
    run = Run(dp, di, m, st[0])
    run.steps(10)
    check("split mode, 10 steps", run, st[10])
    # the host writes the oracle's state at step 10: the split state is formed anew from it
    run.put("P1", st[10]["P1"])
    run.put("S2", st[10]["S2"])
    run.steps(10)
    check("split mode, 10 more steps from a state the host wrote", run, st[20])
    # the eager mode from here: the caller's arrays are brought up to date first
    di.set_mode(0)
    run.steps(10)
    check("eager mode, 10 steps after 20 in split mode", run, st[30])
    assert gpu_lib.gbf_last_status() == abi.GBF_OK
    run.close()


def test_split_mode_media_rewrite_updates_mass_sums(gpu_lib, abi, O, pkg, dropin):
    """The host rewrites the media array after the first step created the
    split domain: the next step reads it in place, and the phase masses the
    drop-in's domain sums (GBF_OUT_MASS on gbf_dropin_domain) take the new
    porosities, as a split domain created with the new media from the same
    state does. The water mass carries the grid's porosity sum over the rows,
    taken from the media: kept from the old media it would be off by percent;
    the two paths differ by the split step's residual (1e-9 bar)."""
    import ctypes
    from importlib import import_module
    Domain = import_module(pkg.__name__ + ".domain").Domain
    dp, di = dropin
    m, st = oracle_states(abi, O, [])
    assert m.m[0] != m.m[1]  # the two media differ in porosity
    di.set_mode(2)
    run = Run(dp, di, m, st[0])
    run.put_media(np.zeros(m.shape, np.int32))
    run.steps(1)
    h = di.domain(run.D.P1)
    assert h and gpu_lib.gbf_domain_set_outputs(h, abi.GBF_OUT_MASS, 8) == abi.GBF_OK
    media1 = (np.random.default_rng(5).random(m.shape) < 0.5).astype(np.int32)
    run.put_media(media1)
    P, S = run.get("P1"), run.get("S2")
    run.steps(1)
    got = np.zeros((8, 2))
    n = ctypes.c_int()
    assert gpu_lib.gbf_domain_mass_history(h, got.ctypes.data, 8, ctypes.byref(n)) == abi.GBF_OK and n.value == 1
    ref = Domain(m, media1, None, None, precision=abi.GBF_PREC_SPLIT)
    ref.set_outputs(abi.GBF_OUT_MASS, 8)
    ref.upload(P, S)
    ref.step(1)
    want = ref.mass_history(1)
    ref.close()
    rel = np.abs(got[0] - want[0]) / np.abs(want[0])
    print(f"\nmedia rewritten: masses {got[0]} vs {want[0]}, relative {rel}")
    assert rel[0] <= 1e-9 and rel[1] <= 1e-4, rel
    assert gpu_lib.gbf_last_status() == abi.GBF_OK
    run.close()


def test_split_mode_parameter_change_forms_the_state_anew(gpu_lib, abi, O, dropin):
    """The compressibilities in consts change between two steps (they enter
    the split state's row densities): the split state is written back to the
    caller's P1, S2 under the old rows and formed anew under the new ones, so
    the run keeps to the fused FP64 mode making the same change (the split
    form's bars). Taken against the old rows, every water-mass defect would be
    off by the change of the row density (about a fifth here)."""
    dp, di = dropin
    m, st = oracle_states(abi, O, [])
    out = {}
    for mode in (2, 1):
        di.set_mode(mode)
        run = Run(dp, di, m, st[0])
        run.steps(10)
        run.c.beta1, run.c.beta2 = 5e-5, 5e-9
        run.steps(10)
        out[mode] = run.get("P1"), run.get("S2")
        assert gpu_lib.gbf_last_status() == abi.GBF_OK
        run.close()
    (Ps, Ss), (Pf, Sf) = out[2], out[1]
    ds, pl2 = float(np.abs(Ss - Sf).max()), rel_l2(Ps, Pf)
    print(f"\nparameters changed after 10 steps: max|dS| {ds:.2e}, rel-L2(P) {pl2:.2e}")
    assert ds <= DS_TOL and pl2 <= P_TOL, (ds, pl2)
