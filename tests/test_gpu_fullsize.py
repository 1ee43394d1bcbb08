"""Parity at the workloads' full sizes, through properties that do not need
the oracle to finish: the measured split forms against the plain FP64 GPU
path (itself pinned to the oracle at 1e-12 by the other tests), ensemble
members against single-domain runs, and run-to-run determinism.

The two full-size workloads:
- config 4: all 256 realizations (edges 48..128 step 16, 208.8M cells), the
  default bench workload, advanced as one ensemble;
- config 2: the 512x512x256 single grid (67.1M cells), the largest one.

Both run at the reference parameter file's compressibilities (1e-4 water,
1e-8 DNAPL: a larger stable dt than the workloads' 1e-9) with 2 kg/s
injected over each grid's top-centre patch, so that the saturation moves by
6e-5 (config 2) to 1e-2 (config 4) in the steps run here (at the workloads' own compressibility it
moves by about 1e-9 a step). Gates, as in the smaller split tests: max |dS| <= 1e-5,
relative L2 of P <= 1e-6, every step's phase masses within 1e-9 (relative)
of the FP64 path's, member by member.
"""
from importlib import import_module

import numpy as np
import pytest

from gpu_util import rel_l2

pytestmark = pytest.mark.gpu

SPLITS = ["split", "split_df", "split_defect"]
DS_TOL = 1e-5
P_TOL = 1e-6
MASS_TOL = 1e-9


def prec(abi, name):
    return {"split": abi.GBF_PREC_SPLIT, "split_df": abi.GBF_PREC_SPLIT_DF, "split_defect": abi.GBF_PREC_SPLIT_DEFECT,
            "f64": abi.GBF_PREC_F64}[name]


def strong(wl, lib, mem):
    """The reference ini's compressibilities and a 2 kg/s injection, at half
    the stable dt of those parameters."""
    mem.model.beta1, mem.model.beta2 = 1e-4, 1e-8
    mem.model.rate = 2.0
    mem.model.newton_tol = 1e-11
    return wl.set_stable_dt(lib, mem, 0.5)


@pytest.fixture(scope="module")
def wl(pkg):
    return import_module(pkg.__name__ + ".workloads")


@pytest.fixture(scope="module")
def config4(gpu_lib, wl):
    return [strong(wl, gpu_lib, m) for m in wl.config4(gpu_lib)]


def run_ensemble(pkg, abi, members, precision, steps):
    E = import_module(pkg.__name__ + ".ensemble").Ensemble
    e = E(members, precision=precision)
    e.set_outputs(abi.GBF_OUT_MASS, steps)
    e.upload_initial()
    e.step(steps)
    e.sync()
    assert e.status() == abi.GBF_OK
    return e


def mass_drift(got, want):
    scale = np.abs(want)
    return float(np.max(np.abs(got - want) / np.where(scale > 0, scale, 1.0)))


def test_config4_full_ensemble_split_forms_match_fp64(gpu_lib, abi, pkg, config4):
    """Every member of the 256-realization ensemble, 30 steps, each split form
    against plain FP64 on the same members."""
    steps = 30
    assert len(config4) == 256 and sum(m.ncells for m in config4) == 208801792
    ref = run_ensemble(pkg, abi, config4, abi.GBF_PREC_F64, steps)
    mr = ref.mass_history(steps)
    assert mr.shape == (steps, 256, 2)
    ref_PS = [(ref.download(r, "P1"), ref.download(r, "S2")) for r in range(len(config4))]
    ref.close()
    moved = max(float(np.abs(S - m.initial_state()[1]).max()) for (_, S), m in zip(ref_PS, config4))
    assert moved > 1e-3, moved  # the saturation front moved
    for form in SPLITS:
        e = run_ensemble(pkg, abi, config4, prec(abi, form), steps)
        md = e.mass_history(steps)
        ds, num, den = 0.0, 0.0, 0.0
        for r, (Pr, Sr) in enumerate(ref_PS):
            Pd, Sd = e.download(r, "P1"), e.download(r, "S2")
            ds = max(ds, float(np.abs(Sd - Sr).max()))
            num += float(np.sum((Pd - Pr) ** 2))
            den += float(np.sum(Pr ** 2))
        e.close()
        assert ds <= DS_TOL, (form, ds)
        assert (num / den) ** 0.5 <= P_TOL, (form, (num / den) ** 0.5)
        assert mass_drift(md, mr) <= MASS_TOL, (form, mass_drift(md, mr))


def test_config4_members_equal_single_domains(gpu_lib, abi, pkg, config4):
    """The smallest member, the first 80-edge member (the ensemble splits its
    columns into k ranges) and the largest one, in the headline form: the
    full ensemble's result equals each member's single-domain run bit for bit."""
    steps = 12
    Domain = import_module(pkg.__name__ + ".domain").Domain
    pick = sorted({min(range(256), key=lambda r: config4[r].ncells),
                   next(r for r in range(256) if config4[r].model.nx == 80),
                   max(range(256), key=lambda r: config4[r].ncells)})
    e = run_ensemble(pkg, abi, config4, abi.GBF_PREC_SPLIT_DEFECT, steps)
    got = {r: (e.download(r, "P1"), e.download(r, "S2")) for r in pick}
    e.close()
    for r in pick:
        mem = config4[r]
        d = Domain(mem.model, mem.media, mem.K, mem.phi, precision=abi.GBF_PREC_SPLIT_DEFECT)
        d.upload(*mem.initial_state())
        d.step(steps)
        assert d.status() == abi.GBF_OK
        P, S = d.download("P1"), d.download("S2")
        d.close()
        assert np.array_equal(P, got[r][0]), (r, mem.model.nx)
        assert np.array_equal(S, got[r][1]), (r, mem.model.nx)


def test_config2_full_grid_split_defect_matches_fp64_and_repeats(gpu_lib, abi, pkg, wl):
    """The 512x512x256 grid, 20 steps: the headline form against plain FP64
    (same gates), and a second run of the headline form from the same start
    giving the same bits (no order-dependent reductions in the state)."""
    steps = 20
    Domain = import_module(pkg.__name__ + ".domain").Domain
    mem = strong(wl, gpu_lib, wl.config2(gpu_lib))
    assert mem.ncells == 512 * 512 * 256
    P0, S0 = mem.initial_state()
    out = []
    for p in (abi.GBF_PREC_F64, abi.GBF_PREC_SPLIT_DEFECT, abi.GBF_PREC_SPLIT_DEFECT):
        d = Domain(mem.model, mem.media, mem.K, mem.phi, precision=p)
        d.set_outputs(abi.GBF_OUT_MASS, steps)
        d.upload(P0, S0)
        d.step(steps)
        assert d.status() == abi.GBF_OK
        out.append((d.download("P1"), d.download("S2"), d.mass_history(steps)))
        d.close()
    (Pr, Sr, mr), (Pd, Sd, md), (Pe, Se, me) = out
    assert float(np.abs(Sr - S0).max()) > 3e-5  # smaller cells, 64 source cells: a slower front (6e-5)
    assert float(np.abs(Sd - Sr).max()) <= DS_TOL
    assert rel_l2(Pd, Pr) <= P_TOL
    assert mass_drift(md, mr) <= MASS_TOL
    assert np.array_equal(Pd, Pe) and np.array_equal(Sd, Se)
    assert np.array_equal(md, me)
