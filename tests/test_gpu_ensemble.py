"""Batched ensembles: every member must equal a single-domain run of the same
model bit for bit (tiling and batching do not change any cell's arithmetic),
for every tile shape and fusion depth, and must match the FP64 oracle to the
precision form's tolerances."""
import ctypes
from dataclasses import dataclass

import numpy as np
import pytest

from gpu_util import p_tol, mass_order_rtol

pytestmark = pytest.mark.gpu


@dataclass
class Mem:
    model: object
    K: np.ndarray = None
    phi: np.ndarray = None
    media: np.ndarray = None

    def initial_state(self):
        m = self.model
        j = np.arange(m.ny, dtype=np.float64)[None, :, None]
        P = np.broadcast_to(m.P_atm + j * m.ro01 * m.g * m.h2, m.shape).copy()
        S = np.zeros(m.shape, np.float64)
        if m.source_mode == 0:
            i, k = np.arange(m.nx), np.arange(m.nz)
            pi = (i >= m.nx // 2 - m.source) & (i <= m.nx // 2 + m.source)
            pk = (k >= m.nz // 2 - m.source) & (k <= m.nz // 2 + m.source)
            S[:, 0, :] = np.where(pk[:, None] & pi[None, :], m.S2_gr, 0.0)
        return P, S


def members(abi, lib):
    """Uneven members: sizes, fields, closures, anisotropy, sources, BCs."""
    out = []
    rng = np.random.default_rng(21)
    # (72, 14, 10): two x tiles of the 64-wide x-pair tile, a 32-wide and a
    # 48-wide one in the mixed shape; (48, 12, 14): one 48x10 tile
    for r, (nx, ny, nz) in enumerate([(24, 20, 18), (36, 16, 22), (16, 16, 16), (40, 24, 12), (72, 14, 10),
                                      (48, 12, 14)]):
        m = abi.reference_model(nx, ny, nz, 1.0)
        m.h1 = m.h2 = m.h3 = 0.05
        m.S_wr[:] = [0.1, 0.1]
        lam = float(rng.uniform(2.0, 3.5))
        m.lam[:] = [lam, lam]
        pd = float(rng.uniform(500, 1500))
        m.P_d[:] = [pd, pd]
        m.kv = float(rng.uniform(0.1, 1.0))
        if r % 2 == 0:
            m.source_mode, m.rate_cells, m.rate = abi.GBF_SOURCE_RATE, 4, float(rng.uniform(1e-3, 1e-2))
            m.bc_mode = abi.GBF_BC_HYDROSTATIC_SIDES
        else:
            m.source = 2
        K = np.empty(m.shape, np.float32)
        phi = np.empty(m.shape, np.float32)
        lib.gbf_fill_lognormal_K(nx, ny, nz, 500 + r, 6.64e-11, float(rng.uniform(0.5, 2.0)), 3.0, K.ctypes.data)
        lib.gbf_fill_porosity(nx, ny, nz, 600 + r, 0.35, 0.05, phi.ctypes.data)
        cells = abi.GbfCells()
        cells.K = K.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        cells.phi = phi.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
        m.dt = 0.5 * lib.gbf_stable_dt(ctypes.byref(m), ctypes.byref(cells), 1.0)
        m.newton_tol = 1e-11
        out.append(Mem(m, K, phi))
    return out


def mods(pkg):
    from importlib import import_module
    return import_module(pkg.__name__ + ".ensemble"), import_module(pkg.__name__ + ".domain")


PRECS = ["f64", "split", "split_df", "split_defect"]


def prec(abi, name):
    return {"split": abi.GBF_PREC_SPLIT, "split_df": abi.GBF_PREC_SPLIT_DF, "split_defect": abi.GBF_PREC_SPLIT_DEFECT,
            "f64": abi.GBF_PREC_F64}[name]


@pytest.mark.parametrize("p", PRECS)
def test_ensemble_members_equal_single_domains(gpu_lib, abi, pkg, p):
    E, D = mods(pkg)
    mems = members(abi, gpu_lib)
    steps = 25
    single = []
    for mem in mems:
        d = D.Domain(mem.model, None, mem.K, mem.phi, precision=prec(abi, p))
        d.set_outputs(abi.GBF_OUT_MASS, steps)
        d.upload(*mem.initial_state())
        d.step(steps)
        single.append((d.download("P1"), d.download("S2"), d.mass_history(steps)))
        d.close()
    shapes = [0] if p == "f64" else [0, 1, 2, 3, 4, 5]  # 3-5: two cells per thread (TMA staging)
    for shape in shapes:
        ens = E.Ensemble(mems, precision=prec(abi, p))
        if p != "f64":
            ens.set_tuning(shape, 0, 0)
            ens.set_tuning(-1, 24, 7)  # a member edge with a short k range (several passes per column)
        ens.set_outputs(abi.GBF_OUT_MASS, steps)
        ens.upload_initial()
        ens.step(steps)
        assert ens.status() == abi.GBF_OK
        mass = ens.mass_history(steps)
        assert mass.shape == (steps, len(mems), 2)
        for r, (P, S, mh) in enumerate(single):
            assert np.array_equal(ens.download(r, "S2"), S), (shape, r)
            assert np.array_equal(ens.download(r, "P1"), P), (shape, r)
            np.testing.assert_allclose(mass[:, r, :], mh, rtol=mass_order_rtol(p, 1e-12), atol=0)
        ens.close()


@pytest.mark.parametrize("p", PRECS)
def test_ensemble_members_match_oracle(gpu_lib, abi, pkg, O, oracle, p):
    E, _ = mods(pkg)
    mems = members(abi, gpu_lib)
    steps = 30
    ens = E.Ensemble(mems, precision=prec(abi, p))
    ens.upload_initial()
    ens.step(steps)
    assert ens.status() == abi.GBF_OK
    for r, mem in enumerate(mems):
        st = O.State(mem.model, None, mem.K, mem.phi)
        P0, S0 = mem.initial_state()
        st["P1"][...] = P0
        st["S2"][...] = S0
        oracle.step(st, steps)
        S, P = ens.download(r, "S2"), ens.download(r, "P1")
        if p == "f64":
            assert np.abs(S - st["S2"]).max() <= 1e-12
            assert np.abs(P - st["P1"]).max() / np.abs(st["P1"]).max() <= p_tol(mem.model)
        else:
            assert np.abs(S - st["S2"]).max() <= 1e-5
            assert np.linalg.norm(P - st["P1"]) / np.linalg.norm(st["P1"]) <= 1e-6
    ens.close()


@pytest.mark.parametrize("p", PRECS)
def test_ensemble_whole_transfers_equal_per_member(gpu_lib, abi, pkg, p):
    """upload_all/download_all (one packed copy each way) equal the per-member
    calls bit for bit, before and after stepping."""
    E, _ = mods(pkg)
    mems = members(abi, gpu_lib)
    a = E.Ensemble(mems, precision=prec(abi, p))
    b = E.Ensemble(mems, precision=prec(abi, p))
    a.upload_initial()
    off = b.offsets()
    P_all = np.concatenate([m.initial_state()[0].ravel() for m in mems])
    S_all = np.concatenate([m.initial_state()[1].ravel() for m in mems])
    b.upload_all(P_all, S_all)
    for ens in (a, b):
        ens.step(7)
    Pb, Sb = np.empty_like(P_all), np.empty_like(S_all)
    b.download_all(Pb, Sb)
    for r, mem in enumerate(mems):
        sl = slice(off[r], off[r + 1])
        assert np.array_equal(a.download(r, "P1").ravel(), Pb[sl])
        assert np.array_equal(a.download(r, "S2").ravel(), Sb[sl])
    a.close()
    b.close()


def test_ensemble_autotune(gpu_lib, abi, pkg):
    E, _ = mods(pkg)
    mems = members(abi, gpu_lib)
    ens = E.Ensemble(mems, precision=abi.GBF_PREC_SPLIT_DF)
    ens.upload_initial()
    tuning = ens.autotune(2)
    assert tuning["tile"] in ("32x8", "64x4", "32x4", "64x8 pairs", "32x16 pairs", "32x16 + 48x10 pairs")
    assert set(tuning["kchunk_by_edge"]) == {m.model.nx for m in mems}
    # after tuning, a fresh run still equals the default-tuned one
    ens.upload_initial()
    ens.step(10)
    ref = E.Ensemble(mems, precision=abi.GBF_PREC_SPLIT_DF)
    ref.upload_initial()
    ref.step(10)
    for r in range(len(mems)):
        assert np.array_equal(ens.download(r, "S2"), ref.download(r, "S2"))
    ens.close()
    ref.close()


@pytest.mark.parametrize("p", ["split", "split_df", "split_defect"])
def test_ensemble_tma_staging_equals_plain_loads(gpu_lib, abi, pkg, p):
    """Persistent ensemble kernel with TMA plane staging (barrier parities
    carried from tile to tile) against plain loads, every tile shape, with a
    short k range so that tiles hold fewer planes than the ring has stages."""
    E, _ = mods(pkg)
    mems = members(abi, gpu_lib)
    steps = 12
    prev = gpu_lib.gbf_set_tma(-1)
    try:
        for shape in (0, 1, 2, 3, 4, 5):
            res = {}
            for tma in (1, 0):
                gpu_lib.gbf_set_tma(tma)
                ens = E.Ensemble(mems, precision=prec(abi, p))
                if shape in (3, 4, 5) and not tma:  # the x-pair tiles have no plain-load form
                    assert gpu_lib.gbf_ensemble_set_tuning(ens.h, shape, 0, 0) == abi.GBF_ERR_ARG
                    gpu_lib.gbf_clear_status()
                    ens.set_tuning(0, 0, 0)
                else:
                    ens.set_tuning(shape, 0, 0)
                ens.set_tuning(-1, 36, 2)
                assert gpu_lib.gbf_ensemble_uses_tma(ens.h) == tma
                ens.upload_initial()
                ens.step(steps)
                assert ens.status() == abi.GBF_OK
                res[tma] = [(ens.download(r, "P1"), ens.download(r, "S2")) for r in range(len(mems))]
                ens.close()
            for r in range(len(mems)):
                assert np.array_equal(res[1][r][0], res[0][r][0]), (shape, r)
                assert np.array_equal(res[1][r][1], res[0][r][1]), (shape, r)
    finally:
        gpu_lib.gbf_set_tma(prev)


@pytest.mark.parametrize("p", PRECS)
def test_ensemble_pinned_transfers_equal_staged(gpu_lib, abi, pkg, p):
    """Page-locked host arrays read and written in place by the conversion
    kernels give the same bits as the copy-staged transfers."""
    import torch
    E, _ = mods(pkg)
    mems = members(abi, gpu_lib)
    cells = sum(m.model.nx * m.model.ny * m.model.nz for m in mems)
    P_all = np.concatenate([m.initial_state()[0].ravel() for m in mems])
    S_all = np.concatenate([m.initial_state()[1].ravel() for m in mems])
    out = {}
    prev = gpu_lib.gbf_set_host_direct(-1)
    try:
        for direct in (1, 0):
            gpu_lib.gbf_set_host_direct(direct)
            Pp = torch.empty(cells, dtype=torch.float64, pin_memory=True).numpy()
            Sp = torch.empty(cells, dtype=torch.float64, pin_memory=True).numpy()
            Pp[...] = P_all
            Sp[...] = S_all
            ens = E.Ensemble(mems, precision=prec(abi, p))
            ens.upload_all(Pp, Sp)
            ens.step(5)
            ens.download_all(Pp, Sp)
            assert ens.status() == abi.GBF_OK
            out[direct] = (Pp.copy(), Sp.copy(), ens.download(2, "S2"))
            ens.close()
    finally:
        gpu_lib.gbf_set_host_direct(prev)
    for a, b in zip(out[1], out[0]):
        assert np.array_equal(a, b)


@pytest.mark.parametrize("p", PRECS)
def test_ensemble_advance_host_equals_three_calls(gpu_lib, abi, pkg, p):
    """The pipelined host-resident call (member groups over three streams)
    equals upload_all + step(n) + download_all bit for bit, with separate and
    with aliased output arrays, and leaves the ensemble in the same state."""
    import torch
    E, _ = mods(pkg)
    mems = members(abi, gpu_lib) * 3  # 15 members: several groups
    cells = sum(m.model.nx * m.model.ny * m.model.nz for m in mems)
    P0 = np.concatenate([m.initial_state()[0].ravel() for m in mems])
    S0 = np.concatenate([m.initial_state()[1].ravel() for m in mems])

    def pinned(a):
        t = torch.empty(a.shape, dtype=torch.float64, pin_memory=True).numpy()
        t[...] = a
        return t

    for nsteps in (1, 4):
        ref = E.Ensemble(mems, precision=prec(abi, p))
        ref.upload_all(P0, S0)
        ref.step(nsteps)
        Pr, Sr = np.empty_like(P0), np.empty_like(S0)
        ref.download_all(Pr, Sr)
        dut = E.Ensemble(mems, precision=prec(abi, p))
        assert gpu_lib.gbf_ensemble_set_pipeline_groups(dut.h, 5) == abi.GBF_OK
        Pi, Si = pinned(P0), pinned(S0)
        Po, So = pinned(np.zeros_like(P0)), pinned(np.zeros_like(S0))
        dut.advance_host(Pi, Si, nsteps, Po, So)
        assert dut.status() == abi.GBF_OK
        assert np.array_equal(Po, Pr) and np.array_equal(So, Sr)
        assert np.array_equal(Pi, P0)  # inputs untouched
        # aliased in/out, pageable arrays
        Pa, Sa = P0.copy(), S0.copy()
        dut.advance_host(Pa, Sa, nsteps)
        assert np.array_equal(Pa, Pr) and np.array_equal(Sa, Sr)
        # the state left behind steps on like the reference ensemble's
        ref.step(2)
        dut.step(2)
        for r in (0, 5, 11):
            assert np.array_equal(dut.download(r, "S2"), ref.download(r, "S2"))
            assert np.array_equal(dut.download(r, "P1"), ref.download(r, "P1"))
        ref.close()
        dut.close()


def test_ensemble_without_tma_refuses_pair_tile(gpu_lib, abi, pkg):
    """A member whose rows are not whole 16-byte units (nx % 4 != 0) rules out
    TMA staging for the ensemble: plain loads, the x-pair tile refused and
    skipped by the autotuner, results still those of single domains."""
    E, D = mods(pkg)
    mems = members(abi, gpu_lib)[:2]
    m = abi.reference_model(18, 12, 10, 1.0)  # nx = 18
    m.h1 = m.h2 = m.h3 = 0.05
    K = np.full(m.shape, 6.64e-11, np.float32)
    phi = np.full(m.shape, 0.35, np.float32)
    cells = abi.GbfCells()
    cells.K = K.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    cells.phi = phi.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    m.dt = 0.5 * gpu_lib.gbf_stable_dt(ctypes.byref(m), ctypes.byref(cells), 1.0)
    mems.append(Mem(m, K, phi))
    ens = E.Ensemble(mems, precision=abi.GBF_PREC_SPLIT_DF)
    assert gpu_lib.gbf_ensemble_uses_tma(ens.h) == 0
    for shape in (3, 4, 5):
        assert gpu_lib.gbf_ensemble_set_tuning(ens.h, shape, 0, 0) == abi.GBF_ERR_ARG
        gpu_lib.gbf_clear_status()
    assert "pairs" not in ens.autotune(1)["tile"]
    ens.upload_initial()
    ens.step(6)
    assert ens.status() == abi.GBF_OK
    d = D.Domain(m, None, K, phi, precision=abi.GBF_PREC_SPLIT_DF)
    d.upload(*mems[2].initial_state())
    d.step(6)
    assert np.array_equal(ens.download(2, "S2"), d.download("S2"))
    assert np.array_equal(ens.download(2, "P1"), d.download("P1"))
    d.close()
    ens.close()
