"""defines.ini (the reference's parameter file, main.cpp:601-684) through
gbf_read_defines: the reference's line rules (CRLF ends, '#' comments in a
single-byte code page, value up to the first space), a path instead of the
fixed Windows path of defines.h:5, and lines the reference cannot handle."""
import ctypes

import pytest

# The keys and values of the reference's own defines.ini, in its layout.
REFERENCE_INI = (
    b"#######################################################################\r\n"
    b"# \xd4\xe0\xe9\xeb \xed\xe0\xf7\xe0\xeb\xfc\xed\xfb\xf5 \xf3\xf1\xeb\xee\xe2\xe8\xe9 NAPL_Filtration #\r\n"
    b"H1=0.02045\r\n#\r\nH2=0.01969\r\n#\r\nH3=0.01969\r\n#\r\nDT=0.001\r\n#\r\n#\r\nTAU=0.002\r\n#\r\n"
    b"L_N=8.528784e-10\r\nL_W=2e-7\r\n#\r\nC=1407\r\n#\r\n#\r\nBETA1=1.0e-4\r\n#\r\nBETA2=1.0e-8\r\n"
    b"#BETA2=1.0e-4\r\n#\r\nNX=15\r\n#\r\nNY=15\r\n#\r\nNZ=15\r\n#\r\nSOURCE=3          \r\n"
    b"SAVE_PLOTS=100000\r\nPRINT_SCREEN=1000\r\nK[0]=6.64e-11\r\nK[1]=7.15e-12\r\nMU1=0.001\r\nMU2=0.0009\r\n"
    b"RO_W=1000\r\nRO_N=1460\r\nLAMBDA[0]=2.7\r\nLAMBDA[1]=2.0\r\nS_WR[0]=0.09\r\nS_WR[1]=0.12\r\nS2_GR=0.4\r\n"
    b"M[0]=0.4\r\nM[1]=0.39\r\nP_D[0]=755\r\nP_D[1]=2060\r\nP_ATM=100000\r\nG_CONST=9.8\r\nOMEGA=1.2\r\n"
    b"EPSILON=1.0e-6\r\n"
)


def read(lib, abi, path):
    m = abi.GbfModel()
    run = abi.GbfRunDefines()
    rc = lib.gbf_read_defines(str(path).encode(), ctypes.byref(m), ctypes.byref(run))
    return rc, m, run


def test_reads_reference_ini_and_matches_reference_constants(pkg, abi, tmp_path):
    lib = pkg.load_library()
    p = tmp_path / "defines.ini"
    p.write_bytes(REFERENCE_INI)
    rc, m, run = read(lib, abi, p)
    assert rc == abi.GBF_OK
    assert (m.nx, m.ny, m.nz, m.source) == (15, 15, 15, 3)
    assert (m.h1, m.h2, m.h3, m.dt, m.beta1, m.beta2) == (0.02045, 0.01969, 0.01969, 0.001, 1e-4, 1e-8)
    assert (run.tau, run.l_w, run.l_n, run.c) == (0.002, 2e-7, 8.528784e-10, 1407.0)
    assert (run.save_plots, run.print_screen) == (100000, 1000)
    # the file's physical constants are the reference's compile-time ones
    ref = abi.reference_model(15, 15, 15, 0.001)
    for f, _ in abi.GbfModel._fields_:
        a, b = getattr(m, f), getattr(ref, f)
        assert (list(a) == list(b)) if hasattr(a, "__len__") else a == b, f


def test_edited_and_untidy_files(pkg, abi, tmp_path):
    lib = pkg.load_library()
    p = tmp_path / "d.ini"
    p.write_bytes(b"\n  \nno equals sign here\nNX = 40 # trailing comment\nNY=30\nNZ=20\n"
                  b"LAMBDA[1]=3.5\nK[0]=1e-12\nP_D[2]=9\nUNKNOWN=1\nDT=0.5")  # no final newline
    rc, m, run = read(lib, abi, p)
    assert rc == abi.GBF_OK
    assert (m.nx, m.ny, m.nz, m.dt) == (40, 30, 20, 0.5)
    assert m.lam[1] == 3.5 and m.K[0] == 1e-12 and list(m.P_d) == [755.0, 2060.0]
    assert lib.gbf_read_defines(str(p).encode(), ctypes.byref(m), None) == abi.GBF_OK


@pytest.mark.parametrize("content", [b"NX=4\nNY=4\n", b"#NX=4\n#NY=4\n#NZ=4\n"])
def test_grid_size_is_required(pkg, abi, tmp_path, content):
    lib = pkg.load_library()
    p = tmp_path / "d.ini"
    p.write_bytes(content)
    assert read(lib, abi, p)[0] == abi.GBF_ERR_ARG
    assert read(lib, abi, tmp_path / "missing.ini")[0] == abi.GBF_ERR_ARG
    lib.gbf_clear_status()
