"""gbf_boundary_f64_noalloc: the boundary pass for callers that cannot
allocate device memory where they apply the boundary conditions (a host loop
that must not stall on cudaMalloc's device synchronisation, a process whose
device memory belongs to another framework's allocator or is budgeted up
front, a driver that hands over only its state arrays). Its scratch is a fixed
device array of the library instead of a caller buffer.

Checked through the C ABI against the allocating entry point
gbf_boundary_f64 on the same inputs, on two calls in a row (the second call
finds the first call's contents in the shared array), within the FP64 test
tolerance. The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import F64_TOL, DevState, assert_field

pytestmark = pytest.mark.gpu


def random_state(O, abi, m, seed):
    rng = np.random.default_rng(seed)
    st = O.State(m, (rng.random(m.shape) < 0.3).astype(np.int32))
    j = np.arange(m.ny, dtype=np.float64)[None, :, None]
    st["P1"][...] = m.P_atm + j * m.ro01 * m.g * m.h2 + rng.uniform(-50.0, 50.0, m.shape)
    st["S2"][...] = rng.uniform(0.0, 0.45, m.shape)
    return st


def test_noalloc_boundary_matches_allocating_entry_point(gpu_lib, abi, O):
    import torch
    lib = gpu_lib
    lib.gbf_boundary_f64_noalloc.restype = ctypes.c_int
    lib.gbf_boundary_f64_noalloc.argtypes = [ctypes.POINTER(abi.GbfModel), abi.GbfArrays, ctypes.c_void_p]
    m = abi.reference_model(40, 36, 32, 0.02)
    m.source = 4
    scratch = torch.empty(lib.gbf_boundary_scratch_doubles(ctypes.byref(m)), dtype=torch.float64, device="cuda")
    for call, seed in enumerate((3, 4)):  # two calls in a row, different inputs
        st = random_state(O, abi, m, seed)
        a, b = DevState(st, abi), DevState(st, abi)
        for ds in (a, b):  # the bottom rule reads the densities of a1
            assert lib.gbf_props_f64(ctypes.byref(m), ds.arrays(), ds.cells(), None) == 0
        assert lib.gbf_boundary_f64(ctypes.byref(m), a.arrays(), ctypes.c_void_p(scratch.data_ptr()), None) == 0
        assert lib.gbf_boundary_f64_noalloc(ctypes.byref(m), b.arrays(), None) == 0
        torch.cuda.synchronize()
        for k in ("P1", "S2"):
            got, want = b.host(k), a.host(k)
            assert_field(k, got, want, tol=F64_TOL)
            assert not np.array_equal(want, st[k]), (call, k)  # the pass changed the faces
    assert lib.gbf_last_status() == abi.GBF_OK
    # sizes beyond its fixed scratch are refused with an error, nothing launched
    big = abi.reference_model(320, 320, 320, 0.02)
    assert lib.gbf_boundary_f64_noalloc(ctypes.byref(big), abi.GbfArrays(), None) == abi.GBF_ERR_ARG
    lib.gbf_clear_status()
