"""gbf_boundary_f64_noalloc: the boundary pass for callers that cannot
allocate device memory where they apply the boundary conditions (a host loop
that must not stall on cudaMalloc's device synchronisation, a process whose
device memory belongs to another framework's allocator or is budgeted up
front, a driver that hands over only its state arrays). Its scratch is a fixed
device array of the library instead of a caller buffer.

Checked through the C ABI against the allocating entry point
gbf_boundary_f64 on the same inputs: both run the same gather and scatter
kernels, so the results must be equal bit for bit. Calls in a row on grids of
decreasing size (each call finds the previous, larger call's contents in the
shared array: a slot the gather missed would show a stale value), then a grid
with exactly the largest boundary the array serves, and one just above it,
which is refused. The file name makes pytest collect it last.
"""
import ctypes

import numpy as np
import pytest

from gpu_util import DevState

pytestmark = pytest.mark.gpu

# the array holds 2^20 doubles: two per boundary cell
LIMIT_CELLS = 524288


def boundary_cells(m):
    return 2 * m.nx * m.ny + 2 * m.nx * (m.nz - 2) + 2 * (m.ny - 2) * (m.nz - 2)


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
    # decreasing boundaries, the last at the array's limit (a 4 x 43690 x 4 column)
    shapes = [(40, 36, 32), (24, 20, 18), (4, 43690, 4)]
    assert boundary_cells(abi.reference_model(*shapes[-1], 0.02)) == LIMIT_CELLS
    for call, (shape, seed) in enumerate(zip(shapes, (3, 4, 5))):
        m = abi.reference_model(*shape, 0.02)
        m.source = 4
        st = random_state(O, abi, m, seed)
        scratch = torch.empty(lib.gbf_boundary_scratch_doubles(ctypes.byref(m)), dtype=torch.float64,
                              device="cuda")
        a, b = DevState(st, abi), DevState(st, abi)
        for ds in (a, b):  # the bottom rule reads the densities of a1
            assert lib.gbf_props_f64(ctypes.byref(m), ds.arrays(), ds.cells(), None) == 0
        assert lib.gbf_boundary_f64(ctypes.byref(m), a.arrays(), ctypes.c_void_p(scratch.data_ptr()), None) == 0
        assert lib.gbf_boundary_f64_noalloc(ctypes.byref(m), b.arrays(), None) == 0
        torch.cuda.synchronize()
        for k in ("P1", "S2"):
            got, want = b.host(k), a.host(k)
            assert np.array_equal(got, want), (call, k, float(np.abs(got - want).max()))
            assert not np.array_equal(want, st[k]), (call, k)  # the pass changed the faces
        del a, b, scratch
    assert lib.gbf_last_status() == abi.GBF_OK
    # one boundary cell pair beyond the array (3 x 65536 x 3: 524290 cells), and
    # a 297^3 cube: refused with an error before anything is launched
    for shape in ((3, 65536, 3), (297, 297, 297)):
        big = abi.reference_model(*shape, 0.02)
        assert boundary_cells(big) > LIMIT_CELLS
        assert lib.gbf_boundary_f64_noalloc(ctypes.byref(big), abi.GbfArrays(), None) == abi.GBF_ERR_ARG
    lib.gbf_clear_status()
