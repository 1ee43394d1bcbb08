"""Pin the oracle (C restatement of cpu.cpp) before trusting it.

1. Against the committed golden fixtures made by running the reference's own
   CPU backend (tests/golden/make_golden.py): bit-exact.
2. Against the reference library itself, when it was built here from the
   reference sources: bit-exact, on more cases.
3. Semantic pins the reference implies (7 Newton iterations, boundary sweep
   order, P_k = 0 in a1, bottom rule reading ro1 at (i,1,0), patch geometry).
"""
import numpy as np
import pytest

from conftest import load_golden


def run_golden(O, oracle, abi, name):
    m, z = load_golden(abi, name)
    st = O.State(m, z["media"].astype(np.int32))
    oracle.initial(st)
    oracle.step(st, int(z["steps"]))
    return st, z


@pytest.mark.parametrize("name", ["ref_run_15cube_dt0.02_100steps.npz",
                                  "ref_run_13x17x19_media_dt0.02_60steps.npz"])
def test_oracle_matches_reference_runs_bit_exact(O, oracle, abi, name):
    st, z = run_golden(O, oracle, abi, name)
    for k in ("P1", "S2", "roS1", "roS2", "u2x", "u2y", "u2z"):
        assert np.array_equal(st[k], z[k]), k
    # the run is not trivial: DNAPL moved into the interior
    assert st["S2"][:, 1:-1, :].max() > 1e-3


def test_oracle_matches_reference_stages_bit_exact(O, oracle, abi):
    m, z = load_golden(abi, "ref_stages_8x9x10.npz")
    st = O.State(m, z["media"].astype(np.int32))
    st["P1"][...] = z["in_P1"]
    st["S2"][...] = z["in_S2"]
    oracle.props(st)
    for k in ("P2", "Xi1", "Xi2", "ro1", "ro2"):
        assert np.array_equal(st[k], z[f"props_{k}"]), k
    oracle.velocity(st)
    for k in ("u1x", "u1y", "u1z", "u2x", "u2y", "u2z"):
        assert np.array_equal(st[k], z[f"velocity_{k}"]), k
    oracle.mass(st)
    for k in ("roS1", "roS2", "roS1_old", "roS2_old"):
        assert np.array_equal(st[k], z[f"mass_{k}"]), k
    oracle.newton(st)
    for k in ("P1", "S2"):
        assert np.array_equal(st[k], z[f"newton_{k}"]), k
    oracle.boundary(st)
    for k in ("P1", "S2"):
        assert np.array_equal(st[k], z[f"boundary_{k}"]), k


@pytest.mark.parametrize("shape,dt,steps,source", [((16, 16, 16), 0.02, 40, 3), ((5, 7, 6), 0.01, 30, 1),
                                                   ((24, 20, 18), 0.02, 25, 4), ((3, 3, 3), 0.02, 5, 0)])
def test_oracle_matches_reference_library(O, oracle, abi, shape, dt, steps, source):
    if not O.Reference.available():
        pytest.skip("reference sources not present on this machine (golden fixtures cover this)")
    ref = O.Reference()
    m = abi.reference_model(*shape, dt)
    m.source = source
    media = (np.random.default_rng(3).random(m.shape) < 0.4).astype(np.int32)
    a, b = O.State(m, media), O.State(m, media)
    ref.initial(a)
    oracle.initial(b)
    ref.step(a, steps)
    oracle.step(b, steps)
    for k in O.ARRAY_ORDER:
        assert np.array_equal(a[k], b[k]), k


def test_newton_runs_reference_iteration_count(O, oracle, abi):
    """7 iterations (defines.h:15): the tolerance stop changes nothing beyond round-off."""
    m, z = load_golden(abi, "ref_stages_8x9x10.npz")
    st = O.State(m, z["media"].astype(np.int32))
    st["P1"][...] = z["in_P1"]
    st["S2"][...] = z["in_S2"]
    oracle.props(st)
    oracle.mass(st)
    one = st.copy()
    one.model = m.copy()
    one.model.newton_iterations = 1
    tol = st.copy()
    tol.model = m.copy()
    tol.model.newton_tol = 1e-9
    oracle.newton(st)
    oracle.newton(one)
    oracle.newton(tol)
    assert np.array_equal(st["S2"], z["newton_S2"])
    # one iteration (the reference GPU kernel's count) is measurably different
    assert np.abs(one["S2"] - st["S2"]).max() > 1e-12
    # converge-and-exit matches the full 7 iterations to round-off
    assert np.abs(tol["S2"] - st["S2"]).max() < 1e-14
    assert np.abs(tol["P1"] - st["P1"]).max() / m.P_atm < 1e-13


def test_boundary_sweep_order_semantics(O, oracle, abi):
    """Edges read the new value of earlier cells in the i->j->k sweep and the
    old value of later ones (cpu.cpp:46-53); S2's j==0 rule falls through to
    the k rules (cpu.cpp:343-362)."""
    m = abi.reference_model(6, 7, 8, 0.01)
    m.source = 1
    rng = np.random.default_rng(5)
    st = O.State(m)
    st["S2"][...] = rng.random(m.shape)
    st["P1"][...] = 1e5 + rng.random(m.shape)
    st["ro1"][...] = 1000 + rng.random(m.shape)
    old = st.copy()
    oracle.boundary(st)
    S, P, S0, P0 = st["S2"], st["P1"], old["S2"], old["P1"]
    nx, ny, nz = m.nx, m.ny, m.nz
    # i == 0 copies the OLD value of (1, j, k), even when that cell is a boundary cell
    assert S[0, 0, 0] == S0[0, 0, 1] and P[3, ny - 1, 0] == P0[3, ny - 1, 1]
    # i == nx-1 copies the NEW value of (nx-2, j, k)
    assert S[0, 0, nx - 1] == S[0, 0, nx - 2] and P[nz - 1, 2, nx - 1] == P[nz - 1, 2, nx - 2]
    # top S: Dirichlet value, then k == 0 copies the OLD (k = 1) value
    assert S[0, 0, 3] == S0[1, 0, 3]
    assert S[4, 0, 3] == m.S2_gr and S[4, 0, 1] == 0.0
    # k == nz-1 at the top copies the NEW Dirichlet value of k = nz-2
    assert S[nz - 1, 0, 2] == S[nz - 2, 0, 2]
    # top P is P_atm (P's j == 0 rule returns before the k rules)
    assert P[0, 0, 3] == m.P_atm
    # bottom P: new P above plus ro1 at (i, 1, 0) times g h2 for every k (cpu.cpp:382)
    i, k = 2, 5
    assert P[k, ny - 1, i] == P[k, ny - 2, i] + old["ro1"][0, 1, i] * m.g * m.h2


def test_props_has_zero_capillary_pressure(O, oracle, abi):
    """a1 sets P2 = P1 (P_k = 0, cpu.cpp:63) while the Newton step uses P_k != 0."""
    m = abi.reference_model(5, 5, 5, 0.01)
    st = O.State(m)
    st["P1"][...] = 123456.0
    st["S2"][...] = 0.3
    oracle.props(st)
    assert np.array_equal(st["P2"], st["P1"])


def test_rate_patch_geometry(oracle, abi):
    import ctypes
    m = abi.reference_model(40, 40, 40, 1e-6)
    m.source_mode, m.rate_cells = abi.GBF_SOURCE_RATE, 3
    cells = [(i, k) for i in range(40) for k in range(40) if oracle.lib.orc_in_rate_patch(ctypes.byref(m), i, k)]
    assert sorted(cells) == [(i, k) for i in (19, 20, 21) for k in (19, 20, 21)]
    m.rate_cells = 8
    cells = [(i, k) for i in range(40) for k in range(40) if oracle.lib.orc_in_rate_patch(ctypes.byref(m), i, k)]
    assert len(cells) == 64 and min(cells) == (16, 16) and max(cells) == (23, 23)


def test_rate_injection_adds_mass(O, oracle, abi):
    """Mass-rate source: per step the interior phase-2 mass grows by rate*dt
    (water-saturated start, nothing leaves in one step)."""
    m = abi.reference_model(12, 12, 12, 1e-3)
    m.source_mode, m.rate_cells, m.rate = abi.GBF_SOURCE_RATE, 2, 1e-4
    m.bc_mode = abi.GBF_BC_HYDROSTATIC_SIDES
    st = O.State(m)
    oracle.initial(st)
    mass = oracle.step(st, 3, want_mass=True)
    assert mass[0, 1] == pytest.approx(1e-4 * 1e-3, rel=1e-9)
    assert st["S2"].max() > 0


def fp32_mobility_drift(abi, O, oracle, lib, case, level=1):
    """Largest relative phase-mass difference per phase over a case's steps
    between the oracle and the oracle at one FP32 experiment level
    (Oracle.fp32_mobilities): 1 its upwinded face mobilities rounded to FP32,
    everything else FP64; 2 the same but the Dirichlet patch's DNAPL faces;
    3 the split forms' FP32 flux arithmetic with FP64 mobilities and the
    patch's DNAPL inflow in FP64; 4 that with FP32 mobilities and the tile's
    FMA-fused minus faces."""
    from test_gpu_f64 import make_case
    out = []
    for lv in (0, level):
        m, st, steps = make_case(abi, O, lib, case)
        m.newton_tol = 0.0
        st.model = m
        oracle.initial(st)
        oracle.fp32_mobilities(lv)
        try:
            out.append(oracle.step(st, steps, want_mass=True))
        finally:
            oracle.fp32_mobilities(0)
    ref, exp = out
    scale = np.where(np.abs(ref) > 0, np.abs(ref), 1.0)
    return (np.abs(exp - ref) / scale).max(axis=0), m


@pytest.mark.parametrize("case", ["reference_ini_16", "reference_odd_5x7x6", "c0_rate_hydrostatic_40",
                                  "heterogeneous_aniso_24x20x18"])
def test_fp32_mobilities_alone_bound_patch_dnapl_mass(abi, O, oracle, pkg, case):
    """Why the DNAPL mass of a Dirichlet-patch run cannot stay within 1e-9 of
    FP64 when face fluxes are FP32: there every kilogram of DNAPL enters
    through the patch faces, so the total inherits the relative rounding of
    the patch cells' mobilities (2^-24 for a correctly rounded FP32 value).
    The oracle with those mobilities alone rounded to FP32 moves the DNAPL
    total by more than 1e-8 in the Dirichlet cases, while water, and both
    phases of the mass-rate cases (whose source is exact), stay at round-off."""
    lib = pkg.load_library()
    drift, m = fp32_mobility_drift(abi, O, oracle, lib, case)
    assert drift[0] <= 1e-10, drift
    if m.source_mode == abi.GBF_SOURCE_DIRICHLET_PATCH:
        assert drift[1] >= 1e-8, drift
    else:
        assert drift[1] <= 1e-12, drift


@pytest.mark.parametrize("case", ["reference_ini_16", "reference_odd_5x7x6", "c0_rate_hydrostatic_40",
                                  "heterogeneous_aniso_24x20x18"])
def test_fp32_flux_stage_bounds_patch_dnapl_mass(abi, O, oracle, pkg, case):
    """What is left of the Dirichlet-patch DNAPL drift once the patch inflow
    is FP64 (the split forms): FP32 mobilities on every other face move the
    DNAPL total by less than 1e-9 (level 2), but the FP32 flux arithmetic
    itself does not stay within it. The patch cells pass on every kilogram
    that enters, and each step rounds their FP32 outflow increments, so the
    total carries a random walk of about 2^-24 / sqrt(patch cells x steps):
    1.05e-9 in the reference parameter file's 16^3 case under correctly
    rounded FP32 with FP64 mobilities (level 3), 1.3e-9 with the tile's FP32
    mobilities and FMA-fused minus faces (level 4). The mass-rate cases, whose
    DNAPL enters through the exact source term, stay at round-off."""
    lib = pkg.load_library()
    d2, m = fp32_mobility_drift(abi, O, oracle, lib, case, 2)
    d3, _ = fp32_mobility_drift(abi, O, oracle, lib, case, 3)
    d4, _ = fp32_mobility_drift(abi, O, oracle, lib, case, 4)
    print(f"\n{case}: DNAPL drift, FP32 mobilities but the patch faces {d2[1]:.2e}, "
          f"FP32 flux arithmetic {d3[1]:.2e}, with FP32 mobilities {d4[1]:.2e}")
    assert max(d2[0], d3[0], d4[0]) <= 1e-9, (d2, d3, d4)
    if m.source_mode == abi.GBF_SOURCE_DIRICHLET_PATCH:
        assert d2[1] <= 1e-9 and d3[1] >= 1e-10 and d4[1] >= 1e-10, (d2, d3, d4)
        if case == "reference_ini_16":
            assert d3[1] > 1e-9 and d4[1] > 1e-9, (d3, d4)
    else:
        assert max(d2[1], d3[1], d4[1]) <= 1e-12, (d2, d3, d4)
