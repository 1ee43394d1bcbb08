"""A GPU domain's Tecplot files (gbf_domain_write_plots) against the files the
library's host writer makes from the oracle's arrays after the same run: same
names and layout, numbers equal to the printed precision."""
import ctypes
import re

import numpy as np
import pytest

from conftest import load_golden
from gpu_util import F64_TOL

pytestmark = pytest.mark.gpu

NUM = re.compile(r"-?\d+\.\d+e[+-]\d+|-?\d+")


def numbers(text):
    return np.array([float(x) for x in NUM.findall(text)])


@pytest.mark.parametrize("prec", ["f64", "split_df", "split_defect"])
def test_domain_plot_files_match_oracle(gpu_lib, abi, pkg, O, oracle, tmp_path, prec):
    from importlib import import_module
    Domain = import_module(pkg.__name__ + ".domain").Domain
    m, z = load_golden(abi, "ref_plots_9x7x5_step4.npz")
    media = np.ascontiguousarray(z["media"], np.int32)
    st = O.State(m)
    oracle.initial(st)
    st.media[...] = media
    P0, S0 = st["P1"].copy(), st["S2"].copy()
    steps = 4
    oracle.step(st, steps)
    t = steps * m.dt
    (tmp_path / "ref").mkdir()
    (tmp_path / "gpu").mkdir()
    arrs = [st[k] for k in ("P1", "S2", "u2x", "u2y", "u2z")]
    assert gpu_lib.gbf_write_plots(str(tmp_path / "ref").encode(), ctypes.byref(m), t,
                                   *[a.ctypes.data for a in arrs], media.ctypes.data) == abi.GBF_OK
    p = {"f64": abi.GBF_PREC_F64, "split_df": abi.GBF_PREC_SPLIT_DF, "split_defect": abi.GBF_PREC_SPLIT_DEFECT}[prec]
    dom = Domain(m, media, precision=p)
    dom.upload(P0, S0)
    dom.step(steps)
    dom.write_plots(tmp_path / "gpu", t)
    ref = {str(q.relative_to(tmp_path / "ref")): q.read_text() for q in (tmp_path / "ref").rglob("*.dat")}
    gpu = {str(q.relative_to(tmp_path / "gpu")): q.read_text() for q in (tmp_path / "gpu").rglob("*.dat")}
    assert set(ref) == set(gpu) and len(ref) == 6
    # printed with 3 significant decimals: a relative 1e-12 state difference can
    # move the last printed digit; the split form differs more in u
    rtol, atol = (2e-3, 1e-12) if prec == "f64" else (2e-2, 1e-5)
    for name in ref:
        a, b = ref[name].splitlines(), gpu[name].splitlines()
        assert a[:3] == b[:3] and len(a) == len(b), name  # headers and line counts
        x, y = numbers("\n".join(a[3:])), numbers("\n".join(b[3:]))
        scale = np.maximum(np.abs(x), 1e-30)
        bad = np.abs(x - y) > rtol * scale + atol
        assert not bad.any(), (name, x[bad][:5], y[bad][:5])
    dom.close()
