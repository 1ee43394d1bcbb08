"""CPU checks of the C ABI library: it loads, exports every symbol the headers
declare, its struct layouts match the bindings, and its host-side logic
(reference constants, stability bound, validation, field generator) is right.
No GPU compute is called."""
import ctypes
import os
import pathlib
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]
# the reference sources (main.cpp, no_communication.cpp, defines.h), named by
# GBF_REFERENCE_DIR; the link test skips where it is unset or they are absent
REF = pathlib.Path(os.environ["GBF_REFERENCE_DIR"]) if os.environ.get("GBF_REFERENCE_DIR") else None


@pytest.fixture(scope="module")
def lib(pkg):
    return pkg.load_library(required=True)


def header_functions(path):
    """Function names declared in a header (return type, name, '(')."""
    text = pathlib.Path(path).read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?[\s\*]([A-Za-z_]\w*)\s*\(", text, flags=re.M)
    return sorted(set(n for n in names if n not in ("if", "sizeof", "defined")))


def test_every_c_symbol_is_exported(lib):
    names = header_functions(ROOT / "include" / "gbflow.h")
    text = (ROOT / "include" / "gbflow.h").read_text()
    assert set(names) == set(re.findall(r"\b(gbf_\w+)\s*\(", text))  # the parser saw every prototype
    assert len(names) >= 29
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_every_dropin_symbol_is_exported(pkg, lib):
    from importlib import import_module
    dropin = import_module(pkg.__name__ + ".dropin")
    names = header_functions(ROOT / "include" / "gbflow_dropin.h")
    cpp = [n for n in names if not n.startswith("gbf_")]
    assert set(cpp) == set(dropin.SYMBOLS), set(cpp) ^ set(dropin.SYMBOLS)
    for n, sym in dropin.SYMBOLS.items():
        assert hasattr(lib, sym), (n, sym)
    for n in names:
        if n.startswith("gbf_"):
            assert hasattr(lib, n), n


def test_struct_layouts(abi, lib):
    assert lib.gbf_abi_sizeof(0) == ctypes.sizeof(abi.GbfModel)
    assert lib.gbf_abi_sizeof(1) == ctypes.sizeof(abi.GbfCells)
    assert lib.gbf_abi_sizeof(2) == ctypes.sizeof(abi.GbfArrays)
    assert lib.gbf_abi_sizeof(3) == ctypes.sizeof(abi.GbfRunDefines)


def test_reference_model_matches_library(abi, lib):
    a = abi.reference_model(15, 16, 17, 0.02)
    b = abi.GbfModel()
    lib.gbf_model_reference(ctypes.byref(b), 15, 16, 17, 0.02)
    assert bytes(a) == bytes(b)


def test_stable_dt(abi, lib):
    # 40^3 unit cube, both compressibilities 1e-9: the explicit scheme is
    # stable at 5e-7 s and not at 1e-6 s (measured with the reference CPU path)
    m = abi.reference_model(40, 40, 40, 1.0)
    m.beta1 = m.beta2 = 1e-9
    m.S_wr[:] = [0.1, 0.1]
    m.h1 = m.h2 = m.h3 = 1.0 / 40
    dt = lib.gbf_stable_dt(ctypes.byref(m), None, 1.0)
    assert 5e-7 < dt < 1e-6
    # the reference ini's compressibilities allow its own dt = 0.02 s
    r = abi.reference_model(40, 40, 40, 0.02)
    assert lib.gbf_stable_dt(ctypes.byref(r), None, 1.0) > 0.02


def test_validate_rejects_bad_models(abi, lib):
    m = abi.reference_model(16, 16, 16, 0.02)
    assert lib.gbf_model_validate(ctypes.byref(m), None, 1) == abi.GBF_OK
    bad = m.copy(); bad.nx = 2
    assert lib.gbf_model_validate(ctypes.byref(bad), None, 0) == abi.GBF_ERR_ARG
    bad = m.copy(); bad.dt = 1e6
    assert lib.gbf_model_validate(ctypes.byref(bad), None, 1) == abi.GBF_ERR_UNSTABLE
    bad = m.copy(); bad.S2_gr = 0.95  # S_e <= 0 on the Dirichlet patch
    assert lib.gbf_model_validate(ctypes.byref(bad), None, 0) == abi.GBF_ERR_ARG
    bad = m.copy(); bad.source_mode = abi.GBF_SOURCE_RATE; bad.rate_cells = 0
    assert lib.gbf_model_validate(ctypes.byref(bad), None, 0) == abi.GBF_ERR_ARG
    media = np.full(m.shape, 2, np.int32)
    cells = abi.GbfCells()
    cells.media = media.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
    assert lib.gbf_model_validate(ctypes.byref(m), ctypes.byref(cells), 0) == abi.GBF_ERR_ARG
    # the largest grid the 32-bit cell offsets allow, and one cell-plane more
    ok = abi.reference_model(1024, 1024, 2047, 0.02)  # 2^31 - 2^20 cells
    assert lib.gbf_model_validate(ctypes.byref(ok), None, 0) == abi.GBF_OK
    big = abi.reference_model(1024, 1024, 2048, 0.02)  # 2^31 cells
    assert lib.gbf_model_validate(ctypes.byref(big), None, 0) == abi.GBF_ERR_ARG
    for dims in ((3, 3, 3), (3, 40, 3)):  # the smallest grids with an interior cell
        assert lib.gbf_model_validate(ctypes.byref(abi.reference_model(*dims, 0.001)), None, 0) == abi.GBF_OK
    for dims in ((0, 16, 16), (16, -1, 16), (16, 16, 2)):
        assert lib.gbf_model_validate(ctypes.byref(abi.reference_model(*dims, 0.02)), None, 0) == abi.GBF_ERR_ARG
    bad = m.copy(); bad.h2 = 0.0
    assert lib.gbf_model_validate(ctypes.byref(bad), None, 0) == abi.GBF_ERR_ARG
    bad = m.copy(); bad.kv = -1.0
    assert lib.gbf_model_validate(ctypes.byref(bad), None, 0) == abi.GBF_ERR_ARG
    K = np.full(m.shape, 6.64e-11, np.float32)
    K[3, 4, 5] = np.nan
    cells = abi.GbfCells()
    cells.K = K.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    assert lib.gbf_model_validate(ctypes.byref(m), ctypes.byref(cells), 0) == abi.GBF_ERR_ARG
    lib.gbf_clear_status()


def test_noalloc_boundary_refuses_grids_beyond_its_array(lib, abi):
    """The allocation-free boundary pass holds 2 doubles per boundary cell in
    its fixed 2^20-double array: at most 524288 boundary cells. The size check
    comes before any device work, so grids just beyond the limit are refused
    here without a GPU (the grids at the limit, 296^3 and a 4 x 43690 x 4
    column with exactly 524288 boundary cells, run in the GPU test)."""
    def nb(m):
        return 2 * m.nx * m.ny + 2 * m.nx * (m.nz - 2) + 2 * (m.ny - 2) * (m.nz - 2)
    assert nb(abi.reference_model(296, 296, 296, 0.02)) == 522152
    assert nb(abi.reference_model(4, 43690, 4, 0.02)) == 524288
    for dims in ((297, 297, 297), (3, 65536, 3), (5, 32767, 5)):  # 525698, 524290, 524290 cells
        m = abi.reference_model(*dims, 0.02)
        assert nb(m) > 524288
        assert lib.gbf_boundary_f64_noalloc(ctypes.byref(m), abi.GbfArrays(), None) == abi.GBF_ERR_ARG
    assert lib.gbf_last_status() == abi.GBF_ERR_ARG
    lib.gbf_clear_status()


def test_standalone_inputs_library_gives_the_same_inputs(lib, abi, O, pkg):
    """libgbf_inputs.so (gbf_fields.cpp built alone, which the timed reference
    CPU run uses so that it does not load libgbflow) makes the same K, phi and
    stable dt as libgbflow, bit for bit, for workloads of every configuration."""
    from importlib import import_module
    wl = import_module(pkg.__name__ + ".workloads")
    inp = O.inputs_library(abi)
    assert inp is not lib
    pairs = [(wl.config0(lib), wl.config0(inp)), (wl.config1(lib, n=40), wl.config1(inp, n=40))]
    pairs += list(zip(wl.config4(lib, members=3), wl.config4(inp, members=3)))
    pairs += list(zip(wl.config3(lib, members=2), wl.config3(inp, members=2)))
    for a, b in pairs:
        assert a.model.dt == b.model.dt and a.model.dt > 0
        for x, y in ((a.K, b.K), (a.phi, b.phi)):
            assert (x is None) == (y is None)
            if x is not None:
                assert np.array_equal(x.view(np.uint32), y.view(np.uint32))


def test_lognormal_field_statistics_and_determinism(lib):
    shape = (48, 40, 32)
    K = np.empty(shape, np.float32)
    assert lib.gbf_fill_lognormal_K(32, 40, 48, 123, 6.64e-11, 1.5, 8.0, K.ctypes.data) == 0
    lk = np.log(K.astype(np.float64)) - np.log(6.64e-11)
    assert abs(lk.mean()) < 1e-6 and abs(lk.std() - 1.5) < 1e-3
    # smoothing: neighbouring cells are strongly correlated (corr length 8 cells)
    c = np.corrcoef(lk[:, :, :-1].ravel(), lk[:, :, 1:].ravel())[0, 1]
    assert c > 0.95
    K2 = np.empty_like(K)
    lib.gbf_fill_lognormal_K(32, 40, 48, 123, 6.64e-11, 1.5, 8.0, K2.ctypes.data)
    assert np.array_equal(K, K2)
    K3 = np.empty_like(K)
    lib.gbf_fill_lognormal_K(32, 40, 48, 124, 6.64e-11, 1.5, 8.0, K3.ctypes.data)
    assert not np.array_equal(K, K3)
    phi = np.empty(shape, np.float32)
    assert lib.gbf_fill_porosity(32, 40, 48, 9, 0.35, 0.05, phi.ctypes.data) == 0
    assert phi.min() >= 0.3 and phi.max() <= 0.4 and abs(phi.mean() - 0.35) < 1e-3


@pytest.mark.skipif(REF is None or not (REF / "main.cpp").exists() or shutil.which("g++") is None,
                    reason="GBF_REFERENCE_DIR unset or the reference sources absent")
def test_dropin_links_with_unmodified_reference_driver(tmp_path):
    """main.cpp and no_communication.cpp, compiled from the reference's own
    sources, link against libgbflow.so in place of gpu.cu (sh/cuda.sh:23-24)."""
    libdir = ROOT / "shmem-cuda-filtration_gb300" / "_build"
    exe = tmp_path / "filtration_gb300"
    cmd = ["g++", "-w", "-O2", f"-I{REF}", str(REF / "main.cpp"), str(REF / "no_communication.cpp"),
           f"-L{libdir}", "-lgbflow", f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    assert exe.exists()
