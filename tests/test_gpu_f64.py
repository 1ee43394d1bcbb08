"""Parity of the plain FP64 GPU paths with the FP64 oracle (cpu.cpp restated).

Every test here calls the CUDA code through the C ABI (libgbflow.so) on
cuda:0 and compares with the oracle on the same inputs. Tolerance: max |dS|
and max-norm relative errors of P and every derived field <= 1e-12 (the
oracle and the kernels differ only in pow/log/exp rounding and in where FMA
contraction happens).
"""
import ctypes

import numpy as np
import pytest

from conftest import load_golden
from gpu_util import F64_TOL, F64_TOL_GRADIENT, DevState, assert_field, p_tol, rel_l2

pytestmark = pytest.mark.gpu


def run_eager_step(lib, m, ds, scratch):
    a, c = ds.arrays(), ds.cells()
    assert lib.gbf_props_f64(ctypes.byref(m), a, c, None) == 0
    assert lib.gbf_velocity_f64(ctypes.byref(m), a, None) == 0
    assert lib.gbf_mass_f64(ctypes.byref(m), a, c, None) == 0
    assert lib.gbf_newton_f64(ctypes.byref(m), a, c, None) == 0
    assert lib.gbf_boundary_f64(ctypes.byref(m), a, ctypes.c_void_p(scratch.data_ptr()), None) == 0


def boundary_scratch(lib, m):
    import torch
    return torch.empty(lib.gbf_boundary_scratch_doubles(ctypes.byref(m)), dtype=torch.float64, device="cuda")


def test_eager_stages_match_reference_fixture(gpu_lib, abi, O):
    """Each of the five kernels, one call each, on a random non-equilibrium
    state with mixed media, against the reference's own stage outputs."""
    lib = gpu_lib
    m, z = load_golden(abi, "ref_stages_8x9x10.npz")
    st = O.State(m, z["media"].astype(np.int32))
    st["P1"][...] = z["in_P1"]
    st["S2"][...] = z["in_S2"]
    ds = DevState(st, abi)
    a, c = ds.arrays(), ds.cells()
    assert lib.gbf_props_f64(ctypes.byref(m), a, c, None) == 0
    for k in ("P2", "Xi1", "Xi2", "ro1", "ro2"):
        assert_field(k, ds.host(k), z[f"props_{k}"])
    assert lib.gbf_velocity_f64(ctypes.byref(m), a, None) == 0
    for k in ("u1x", "u1y", "u1z", "u2x", "u2y", "u2z"):
        assert_field(k, ds.host(k), z[f"velocity_{k}"])
    assert lib.gbf_mass_f64(ctypes.byref(m), a, c, None) == 0
    for k in ("roS1", "roS2", "roS1_old", "roS2_old"):
        assert_field(k, ds.host(k), z[f"mass_{k}"])
    assert lib.gbf_newton_f64(ctypes.byref(m), a, c, None) == 0
    for k in ("P1", "S2"):
        assert_field(k, ds.host(k), z[f"newton_{k}"])
    scratch = boundary_scratch(lib, m)
    assert lib.gbf_boundary_f64(ctypes.byref(m), a, ctypes.c_void_p(scratch.data_ptr()), None) == 0
    for k in ("P1", "S2"):
        assert_field(k, ds.host(k), z[f"boundary_{k}"])


@pytest.mark.parametrize("name", ["ref_run_15cube_dt0.02_100steps.npz",
                                  "ref_run_13x17x19_media_dt0.02_60steps.npz"])
def test_eager_runs_match_reference_fixture(gpu_lib, abi, O, oracle, name):
    m, z = load_golden(abi, name)
    st = O.State(m, z["media"].astype(np.int32))
    oracle.initial(st)
    ds = DevState(st, abi)
    scratch = boundary_scratch(gpu_lib, m)
    for _ in range(int(z["steps"])):
        run_eager_step(gpu_lib, m, ds, scratch)
    for k in ("P1", "S2", "roS1", "roS2", "u2x", "u2y", "u2z"):
        assert_field(k, ds.host(k), z[k])


def make_case(abi, O, lib, case):
    """Models of the parity cases, with their cell fields and initial state."""
    if case == "reference_ini_16":
        m = abi.reference_model(16, 16, 16, 0.02)
        st = O.State(m)
        steps = 60
    elif case == "reference_odd_5x7x6":
        m = abi.reference_model(5, 7, 6, 0.01)
        m.source = 1
        st = O.State(m, (np.random.default_rng(2).random(m.shape) < 0.5).astype(np.int32))
        steps = 40
    elif case == "c0_rate_hydrostatic_40":
        # 1 m cube, 40^3, beta = 1e-9 for both phases, DNAPL at 1e-4 kg/s into
        # the top-centre 3x3 cells, hydrostatic sides, no-flow bottom.
        m = abi.reference_model(40, 40, 40, 1.0)
        m.h1 = m.h2 = m.h3 = 1.0 / 40
        m.beta1 = m.beta2 = 1e-9
        m.S_wr[:] = [0.1, 0.1]
        m.source_mode, m.rate_cells, m.rate = abi.GBF_SOURCE_RATE, 3, 1e-4
        m.bc_mode = abi.GBF_BC_HYDROSTATIC_SIDES
        m.dt = 0.5 * lib.gbf_stable_dt(ctypes.byref(m), None, 1.0)
        st = O.State(m)
        steps = 40
    elif case == "heterogeneous_aniso_24x20x18":
        m = abi.reference_model(24, 20, 18, 1.0)
        m.h1 = m.h2 = m.h3 = 0.05
        m.S_wr[:] = [0.1, 0.1]
        m.lam[:] = [2.3, 2.3]
        m.P_d[:] = [900.0, 900.0]
        m.kv = 0.4
        m.source_mode, m.rate_cells, m.rate = abi.GBF_SOURCE_RATE, 4, 2e-3
        m.bc_mode = abi.GBF_BC_HYDROSTATIC_SIDES
        K = np.empty(m.shape, np.float32)
        phi = np.empty(m.shape, np.float32)
        assert lib.gbf_fill_lognormal_K(m.nx, m.ny, m.nz, 77, 6.64e-11, 1.0, 3.0, K.ctypes.data) == 0
        assert lib.gbf_fill_porosity(m.nx, m.ny, m.nz, 78, 0.35, 0.05, phi.ctypes.data) == 0
        st = O.State(m, None, K, phi)
        cells = st.gbf_cells(abi)
        m.dt = 0.5 * lib.gbf_stable_dt(ctypes.byref(m), ctypes.byref(cells), 1.0)
        steps = 80
    else:
        raise KeyError(case)
    return m, st, steps


CASES = ["reference_ini_16", "reference_odd_5x7x6", "c0_rate_hydrostatic_40", "heterogeneous_aniso_24x20x18"]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("newton_tol", [0.0, 1e-11])
def test_domain_f64_matches_oracle(gpu_lib, abi, O, oracle, pkg, case, newton_tol):
    """Fused FP64 domain (props pass, flux+Newton pass, face pass) against the
    oracle, with the reference's 7 Newton iterations and with converge-and-exit."""
    from importlib import import_module
    Domain = import_module(pkg.__name__ + ".domain").Domain
    m, st, steps = make_case(abi, O, gpu_lib, case)
    m.newton_tol = newton_tol
    st.model = m
    oracle.initial(st)
    P0, S0 = st["P1"].copy(), st["S2"].copy()
    dom = Domain(m, st.media, st.K, st.phi)
    dom.set_outputs(abi.GBF_OUT_MASS, steps)
    dom.upload(P0, S0)
    ref_mass = oracle.step(st, steps, want_mass=True)
    dom.step(steps)
    assert dom.status() == abi.GBF_OK
    P, S = dom.download("P1"), dom.download("S2")
    assert_field("S2", S, st["S2"])
    assert_field("P1", P, st["P1"], tol=p_tol(m))
    assert rel_l2(P, st["P1"]) <= p_tol(m)
    assert np.abs(st["S2"] - S0).max() > 1e-8, "case does not move the saturation"
    mass = dom.mass_history(steps)
    assert mass.shape == (steps, 2)
    for ph in range(2):
        scale = np.abs(ref_mass[:, ph]).max()
        if scale > 0:
            assert np.abs(mass[:, ph] - ref_mass[:, ph]).max() <= 1e-12 * scale, ph
    dom.close()


@pytest.mark.parametrize("mode", [0, 1])
def test_dropin_functions_match_oracle(gpu_lib, abi, O, oracle, pkg, mode):
    """The defines.h function set exactly as main.cpp drives it (allocation,
    H->D loads, time_step_function's five calls, D->H loads), eager (0) and
    fused (1) modes, against the oracle."""
    from importlib import import_module
    dp = import_module(pkg.__name__ + ".dropin")
    di = dp.DropIn()
    di.set_mode(mode)
    m = abi.reference_model(16, 14, 12, 0.02)
    m.source = 2
    media = (np.random.default_rng(4).random(m.shape) < 0.25).astype(np.int32)
    st = O.State(m, media)
    oracle.initial(st)
    c = dp.consts_from_model(m)
    H, D = dp.PtrArrays(), dp.PtrArrays()
    bX, bY, bZ = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    di.f["Device_Initialize"](0, ctypes.byref(bX), ctypes.byref(bY), ctypes.byref(bZ), m.nx, c)
    buf = ctypes.c_void_p()
    di.f["device_memory_alloc"](ctypes.byref(D), ctypes.byref(buf), m.nx + 3, c)
    assert gpu_lib.gbf_last_status() == 0
    for name in ("P1", "S2", "roS1_old", "roS2_old"):
        di.f["load_data_to_device"](st[name].ctypes.data, getattr(D, name), m.nx, c)
    di.f["load_data_to_device_int"](st.media.ctypes.data, D.media, m.nx, c)
    steps = 30
    oracle.step(st, steps)
    for s in range(1, steps + 1):
        di.time_step(H, D, c, s * m.dt, bX.value, bY.value, bZ.value)
    for name in ("P1", "S2", "u2x", "u2y", "u2z", "roS1", "roS2", "roS1_old", "roS2_old", "Xi1", "Xi2", "ro1",
                 "ro2", "P2", "u1x", "u1y", "u1z"):
        out = np.empty(m.shape, np.float64)
        di.f["load_data_to_host"](out.ctypes.data, getattr(D, name), m.nx, c)
        tol = F64_TOL_GRADIENT if (mode == 1 and name.startswith("u")) else F64_TOL
        assert_field(name, out, st[name], tol=tol)
    # a1 alone after the steps: its arrays follow the latest state, the
    # velocities keep the last step's values (fused mode materialises them first)
    di.f["ro_P2_Xi_calculation"](H, D, c, m.nx, 0, 1, bX.value, bY.value, bZ.value)
    st2 = st.copy()
    oracle.props(st2)
    for name, ref in (("P2", st2["P2"]), ("Xi1", st2["Xi1"]), ("u2x", st["u2x"]), ("roS2_old", st["roS2_old"])):
        out = np.empty(m.shape, np.float64)
        di.f["load_data_to_host"](out.ctypes.data, getattr(D, name), m.nx, c)
        assert_field(name, out, ref, tol=F64_TOL_GRADIENT if name.startswith("u") else F64_TOL)
    assert gpu_lib.gbf_last_status() == 0
    di.f["device_memory_free"](D, buf)
    di.set_mode(0)


def test_nonfinite_state_sets_device_status(gpu_lib, abi, O, oracle, pkg):
    """A NaN in the host input reaches the device and raises the non-finite
    status after the step (read on the host; the context stays usable)."""
    from importlib import import_module
    Domain = import_module(pkg.__name__ + ".domain").Domain
    m = abi.reference_model(12, 12, 12, 0.01)
    st = O.State(m)
    oracle.initial(st)
    S = st["S2"].copy()
    S[6, 6, 6] = np.nan
    dom = Domain(m)
    dom.upload(st["P1"], S)
    dom.step(2)
    assert dom.status() == abi.GBF_ERR_NONFINITE
    gpu_lib.gbf_clear_status()
    dom.upload(st["P1"], st["S2"])
    dom.step(2)
    assert dom.status() == abi.GBF_OK
    dom.close()
