"""GPU domains write and read checkpoints in the reference's save/save.dat
layout: a file written by the reference's own save() restores into an FP64
and a split domain and the runs continue like the oracle's; a domain's
checkpoint carries its state and the reference's roS1_old/roS2_old."""
import ctypes

import numpy as np
import pytest

from gpu_util import F64_TOL, p_tol
from test_checkpoint import golden_file, read

pytestmark = pytest.mark.gpu


def domain_cls(pkg):
    from importlib import import_module
    return import_module(pkg.__name__ + ".domain").Domain


@pytest.mark.parametrize("prec", ["f64", "split_df", "split_defect"])
def test_reference_checkpoint_restores_into_domain(gpu_lib, abi, pkg, O, oracle, tmp_path, prec):
    m, steps, path = golden_file(abi, tmp_path)
    rc, step, got, media = read(gpu_lib, m, path)
    assert rc == abi.GBF_OK
    p = {"f64": abi.GBF_PREC_F64, "split_df": abi.GBF_PREC_SPLIT_DF, "split_defect": abi.GBF_PREC_SPLIT_DEFECT}[prec]
    dom = domain_cls(pkg)(m, media, precision=p)
    assert dom.restore(path) == steps
    more = 10
    dom.step(more)
    assert dom.status() == abi.GBF_OK
    st = O.State(m, media)
    st["P1"][...] = got["P1"]
    st["S2"][...] = got["S2"]
    oracle.step(st, more)
    S, P = dom.download("S2"), dom.download("P1")
    if prec == "f64":
        assert np.abs(S - st["S2"]).max() <= F64_TOL
        assert np.abs(P - st["P1"]).max() / np.abs(st["P1"]).max() <= p_tol(m)
    else:
        assert np.abs(S - st["S2"]).max() <= 1e-5
    # a file with other media is refused
    dom2 = domain_cls(pkg)(m, 1 - media, precision=p)
    with pytest.raises(RuntimeError):
        dom2.restore(path)
    gpu_lib.gbf_clear_status()
    dom.close()
    dom2.close()


def test_domain_checkpoint_carries_state_and_old_masses(gpu_lib, abi, pkg, O, oracle, tmp_path):
    """After n steps the file holds the domain's P1, S2 bit for bit and the
    start-of-step masses of step n (the oracle's roS1_old, roS2_old)."""
    m, steps, path = golden_file(abi, tmp_path)
    rc, step, got, media = read(gpu_lib, m, path)
    dom = domain_cls(pkg)(m, media)
    dom.upload(got["P1"], got["S2"])
    out = tmp_path / "dom.dat"
    dom.save(out, 0)  # before a step: old masses are zeros
    rc, j, c0, md0 = read(gpu_lib, m, out)
    assert rc == abi.GBF_OK and j == 0 and not c0["roS1_old"].any()
    assert np.array_equal(c0["P1"], got["P1"]) and np.array_equal(md0, media)
    dom.step(6)
    dom.save(out, steps + 6)
    rc, j, c, md = read(gpu_lib, m, out)
    assert rc == abi.GBF_OK and j == steps + 6
    assert np.array_equal(c["P1"], dom.download("P1")) and np.array_equal(c["S2"], dom.download("S2"))
    st = O.State(m, media)
    st["P1"][...] = got["P1"]
    st["S2"][...] = got["S2"]
    oracle.step(st, 6)
    bnd = np.ones(m.shape, bool)
    bnd[1:-1, 1:-1, 1:-1] = False
    for k in ("roS1_old", "roS2_old"):
        ref = st[k]
        assert np.abs(c[k] - ref).max() <= 1e-12 * np.abs(ref).max(), k
        assert not c[k][bnd].any() and not ref[bnd].any(), k  # boundary cells carry no old masses
    dom.close()


def test_split_checkpoint_round_trip(gpu_lib, abi, pkg, tmp_path):
    """A split domain's checkpoint restores into a fresh split domain; its run
    stays within the split form's saturation bar of the uninterrupted run."""
    from importlib import import_module
    wl = import_module(pkg.__name__ + ".workloads")
    mem = wl.config1(gpu_lib, n=48, seed=9)
    wl.set_stable_dt(gpu_lib, mem, 0.5)
    Domain = domain_cls(pkg)
    a = Domain(mem.model, None, mem.K, mem.phi, precision=abi.GBF_PREC_SPLIT_DF)
    a.upload(*mem.initial_state())
    a.step(20)
    out = tmp_path / "split.dat"
    a.save(out, 20)
    b = Domain(mem.model, None, mem.K, mem.phi, precision=abi.GBF_PREC_SPLIT_DF)
    assert b.restore(out) == 20
    assert np.array_equal(b.download("S2"), a.download("S2"))
    a.step(20)
    b.step(20)
    assert a.status() == abi.GBF_OK and b.status() == abi.GBF_OK
    assert np.abs(a.download("S2") - b.download("S2")).max() <= 1e-5
    a.close()
    b.close()
