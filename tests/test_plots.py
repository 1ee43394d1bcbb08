"""Tecplot output of the reference's save_data_plots (main.cpp:319-482): the
library's writer produces the reference's files byte for byte from the same
arrays (tests/golden/ref_plots_9x7x5_step4.npz, written by the reference's
own function)."""
import ctypes

import numpy as np

from conftest import load_golden

NAME = "ref_plots_9x7x5_step4.npz"


def write(lib, m, d, t, z):
    arrs = [np.ascontiguousarray(z[k], np.float64) for k in ("P1", "S2", "u2x", "u2y", "u2z")]
    media = np.ascontiguousarray(z["media"], np.int32)
    rc = lib.gbf_write_plots(str(d).encode(), ctypes.byref(m), t, *[a.ctypes.data for a in arrs], media.ctypes.data)
    return rc


def test_writer_reproduces_reference_plot_files(pkg, abi, tmp_path):
    lib = pkg.load_library()
    m, z = load_golden(abi, NAME)
    t = float(z["t"])
    assert write(lib, m, tmp_path, t, z) == abi.GBF_OK
    ref_files = {k[5:]: bytes(z[k]) for k in z.files if k.startswith("file:")}
    mine = {str(p.relative_to(tmp_path)): p.read_bytes() for p in tmp_path.rglob("*.dat")}
    assert set(mine) == set(ref_files)
    for name, data in ref_files.items():
        assert mine[name] == data, name
    # the run is not trivial: DNAPL entered and moves
    assert np.abs(z["u2y"]).max() > 0 and z["S2"].max() > 0


def test_writer_refuses_bad_arguments(pkg, abi, tmp_path):
    lib = pkg.load_library()
    m, z = load_golden(abi, NAME)
    assert lib.gbf_write_plots(None, ctypes.byref(m), 0.0, None, None, None, None, None, None) == abi.GBF_ERR_ARG
    assert write(lib, m, tmp_path / "missing" / "deeper", 0.0, z) == abi.GBF_ERR_ARG
    lib.gbf_clear_status()
