"""gbf_domain_advance_host: one step of a single grid from host FP64 arrays to
host FP64 arrays, pipelined over slabs of planes (the copy engines move one
slab in and another out while the compute stream converts, steps and
converts back a third; grids of 2M cells or more, slabs of about 1M cells).
Its state must equal upload + step + download bit for
bit; its step's phase masses, the same cells summed in other partial blocks,
agree to 1e-11 (a small DNAPL total is the difference of large sums, so the
blocks' 2^-48 roundings weigh up to a few hundred times more in it: 4e-13
measured); its CFL numbers (maxima) are equal. Covered: the x-pair TMA tile (a
grid with K and porosity fields, 160^3: three slabs), the plain-load tile (a
media table, 200x160x130, three slabs of uneven depth), two slabs of four
planes (512x512x10), every split form, outputs in place and apart, pageable
and page-locked host arrays, repeated calls on the pipeline's buffers, and the
calls that are not pipelined (a Dirichlet patch, FP64, several steps, a grid
below 2M cells).
"""
from importlib import import_module

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FORMS = ["split", "split_df", "split_defect"]


def prec(abi, form):
    return {"split": abi.GBF_PREC_SPLIT, "split_df": abi.GBF_PREC_SPLIT_DF, "split_defect": abi.GBF_PREC_SPLIT_DEFECT,
            "f64": abi.GBF_PREC_F64}[form]


def field_grid(pkg, lib, n=160):
    """Config 1's heterogeneous rate-injection grid at n^3 (TMA x-pair tile),
    at the reference ini's compressibilities so that the step moves S."""
    wl = import_module(pkg.__name__ + ".workloads")
    mem = wl.config1(lib, n=n, seed=4321)
    mem.model.beta1, mem.model.beta2 = 1e-4, 1e-8
    mem.model.rate = 2.0
    wl.set_stable_dt(lib, mem, 0.5)
    mem.model.newton_tol = 1e-11
    return mem.model, None, mem.K, mem.phi, mem.initial_state()


def media_grid(abi, O, shape, source_mode, seed):
    """A media-table grid (plain-load tile): mixed media, a perturbed
    hydrostatic state with some DNAPL."""
    m = abi.reference_model(*shape, 0.02)
    rng = np.random.default_rng(seed)
    media = (rng.random(m.shape) < 0.4).astype(np.int32)
    if source_mode == "rate":
        m.source_mode, m.rate_cells, m.rate = abi.GBF_SOURCE_RATE, 2, 1e-3
        m.bc_mode = abi.GBF_BC_HYDROSTATIC_SIDES
    j = np.arange(m.ny, dtype=np.float64)[None, :, None]
    P = m.P_atm + j * m.ro01 * m.g * m.h2 + rng.uniform(-20.0, 20.0, m.shape)
    S = rng.uniform(0.0, 0.3, m.shape)
    return m, media, None, None, (P, S)


def run_pair(abi, pkg, grid, form, pinned=False, inplace=True, calls=1, nsteps=1, flags=None):
    Domain = import_module(pkg.__name__ + ".domain").Domain
    m, media, K, phi, (P0, S0) = grid
    flags = abi.GBF_OUT_MASS if flags is None else flags
    ref = Domain(m, media, K, phi, precision=prec(abi, form))
    ref.set_outputs(flags, 8)
    dut = Domain(m, media, K, phi, precision=prec(abi, form))
    dut.set_outputs(flags, 8)
    if pinned:
        import torch
        P = torch.empty(P0.shape, dtype=torch.float64, pin_memory=True).numpy()
        S = torch.empty(S0.shape, dtype=torch.float64, pin_memory=True).numpy()
        P[...] = P0
        S[...] = S0
    else:
        P, S = P0.copy(), S0.copy()
    Pr, Sr = P0.copy(), S0.copy()
    for _ in range(calls):
        ref.upload(Pr, Sr)
        ref.step(nsteps)
        Pr, Sr = ref.download("P1"), ref.download("S2")
        if inplace:
            dut.advance_host(P, S, nsteps)
        else:
            Po, So = np.empty_like(P0), np.empty_like(S0)
            dut.advance_host(P, S, nsteps, Po, So)
            P, S = Po, So
    assert ref.status() == abi.GBF_OK and dut.status() == abi.GBF_OK
    out = {"P": (np.asarray(P), Pr), "S": (np.asarray(S), Sr),
           "mass": (dut.mass_history(nsteps), ref.mass_history(nsteps))}
    if flags & abi.GBF_OUT_CFL:
        out["cfl"] = (dut.cfl_history(nsteps), ref.cfl_history(nsteps))
    ref.close()
    dut.close()
    return out


def check(out, moved=None):
    for k in ("P", "S"):
        got, want = out[k]
        assert np.array_equal(got, want), (k, float(np.abs(got - want).max()))
    got, want = out["mass"]
    assert got.shape == want.shape and np.all(np.isfinite(got))
    assert np.max(np.abs(got - want) / np.abs(want)) <= 1e-11, (got, want)
    if "cfl" in out:
        assert np.array_equal(*out["cfl"])
    if moved is not None:
        assert np.abs(out["S"][1] - moved).max() > 0  # the step did something


@pytest.mark.parametrize("form", FORMS)
def test_pipelined_step_equals_three_calls_tma_tile(gpu_lib, abi, pkg, form):
    grid = field_grid(pkg, gpu_lib)
    out = run_pair(abi, pkg, grid, form, flags=abi.GBF_OUT_MASS | abi.GBF_OUT_CFL)
    check(out, moved=grid[4][1])


@pytest.mark.parametrize("form", FORMS)
def test_pipelined_step_equals_three_calls_media_table(gpu_lib, abi, O, pkg, form):
    grid = media_grid(abi, O, (200, 160, 130), "rate", 7)
    check(run_pair(abi, pkg, grid, form, inplace=False), moved=grid[4][1])


def test_pipelined_step_two_thin_slabs_pinned_and_repeated(gpu_lib, abi, O, pkg):
    check(run_pair(abi, pkg, media_grid(abi, O, (512, 512, 10), "rate", 8), "split", pinned=True))
    check(run_pair(abi, pkg, field_grid(pkg, gpu_lib, n=128), "split", pinned=True, calls=3))


@pytest.mark.parametrize("case", ["patch", "f64", "steps", "small"])
def test_calls_not_pipelined_equal_three_calls(gpu_lib, abi, O, pkg, case):
    if case == "patch":
        out = run_pair(abi, pkg, media_grid(abi, O, (30, 18, 22), "patch", 9), "split")
    elif case == "f64":
        out = run_pair(abi, pkg, media_grid(abi, O, (30, 18, 22), "rate", 10), "f64")
    elif case == "steps":
        out = run_pair(abi, pkg, field_grid(pkg, gpu_lib, n=128), "split", nsteps=3)
    else:
        out = run_pair(abi, pkg, field_grid(pkg, gpu_lib, n=48), "split")
    for k in ("P", "S"):
        assert np.array_equal(*out[k]), k
    assert np.array_equal(*out["mass"])
