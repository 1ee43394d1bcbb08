"""Checkpoint files in the reference's save/save.dat layout (main.cpp:485-572),
host side: the library's reader and writer against a file written by the
reference's own save() (tests/golden/ref_checkpoint_10x8x6_step7.npz), and
against the oracle's state after the same run (bit-exact)."""
import ctypes

import numpy as np
import pytest

from conftest import load_golden

NAME = "ref_checkpoint_10x8x6_step7.npz"


def golden_file(abi, tmp_path):
    m, z = load_golden(abi, NAME)
    path = tmp_path / "save.dat"
    path.write_bytes(z["dat"].tobytes())
    return m, int(z["steps"]), path


def read(lib, m, path):
    out = {k: np.empty(m.shape, np.float64) for k in ("P1", "S2", "roS1_old", "roS2_old")}
    media = np.empty(m.shape, np.int32)
    step = ctypes.c_int(-1)
    rc = lib.gbf_checkpoint_read(str(path).encode(), ctypes.byref(m), ctypes.byref(step), out["P1"].ctypes.data,
                                 out["S2"].ctypes.data, out["roS1_old"].ctypes.data, out["roS2_old"].ctypes.data,
                                 media.ctypes.data)
    return rc, step.value, out, media


def test_reads_reference_checkpoint(pkg, abi, O, oracle, tmp_path):
    lib = pkg.load_library()
    m, steps, path = golden_file(abi, tmp_path)
    assert path.stat().st_size == lib.gbf_checkpoint_bytes(ctypes.byref(m))
    rc, step, got, media = read(lib, m, path)
    assert rc == abi.GBF_OK and step == steps
    # the same run through the oracle (bit-exact with the reference's cpu.cpp)
    st = O.State(m)
    oracle.initial(st)
    st.media[...] = media  # the run's media were set after initial_data
    oracle.step(st, steps)
    for k in ("P1", "S2", "roS1_old", "roS2_old"):
        assert np.array_equal(got[k], st[k]), k
    assert media.any() and (media != 0).sum() < media.size  # mixed media travelled
    assert np.abs(st["roS2_old"]).max() > 0                 # DNAPL masses are in the file


def test_writer_reproduces_reference_bytes(pkg, abi, tmp_path):
    lib = pkg.load_library()
    m, steps, path = golden_file(abi, tmp_path)
    rc, step, got, media = read(lib, m, path)
    assert rc == abi.GBF_OK
    mine = tmp_path / "mine.dat"
    assert lib.gbf_checkpoint_write(str(mine).encode(), ctypes.byref(m), step, got["P1"].ctypes.data,
                                    got["S2"].ctypes.data, got["roS1_old"].ctypes.data,
                                    got["roS2_old"].ctypes.data, media.ctypes.data) == abi.GBF_OK
    assert mine.read_bytes() == path.read_bytes()


def test_rejects_other_grids(pkg, abi, tmp_path):
    lib = pkg.load_library()
    m, steps, path = golden_file(abi, tmp_path)
    other = m.copy()
    other.nx += 1  # size mismatch
    assert read(lib, other, path)[0] == abi.GBF_ERR_ARG
    other = m.copy()
    other.nx, other.ny = m.ny, m.nx  # same size, other coordinates
    assert read(lib, other, path)[0] == abi.GBF_ERR_ARG
    other = m.copy()
    other.h1 *= 2.0
    assert read(lib, other, path)[0] == abi.GBF_ERR_ARG
    assert read(lib, m, tmp_path / "missing.dat")[0] == abi.GBF_ERR_ARG
    lib.gbf_clear_status()


def test_reference_restore_reads_library_file(pkg, abi, O, oracle, tmp_path):
    """The reference's own restore() (main.cpp:541) reads a file the library
    wrote, and its run continues exactly like the oracle's."""
    if not O.Reference.available():
        pytest.skip("reference library not built (reference sources absent)")
    lib = pkg.load_library()
    m, steps, path = golden_file(abi, tmp_path)
    rc, step, got, media = read(lib, m, path)
    (tmp_path / "run" / "save").mkdir(parents=True)
    out = tmp_path / "run" / "save" / "save.dat"
    assert lib.gbf_checkpoint_write(str(out).encode(), ctypes.byref(m), 11, got["P1"].ctypes.data,
                                    got["S2"].ctypes.data, None, None, media.ctypes.data) == abi.GBF_OK
    ref = O.Reference()
    st = O.State(m, np.zeros(m.shape, np.int32))
    assert ref.restore(st, tmp_path / "run") == 11
    assert np.array_equal(st["P1"], got["P1"]) and np.array_equal(st.media, media)
    ref.step(st, 3)
    orc = O.State(m, media)
    orc["P1"][...] = got["P1"]
    orc["S2"][...] = got["S2"]
    oracle.step(orc, 3)
    assert np.array_equal(st["S2"], orc["S2"]) and np.array_equal(st["P1"], orc["P1"])
