"""ctypes mirror of include/gbflow.h and the loader of the in-tree libgbflow.so.

The library is the product: a missing library on a GPU machine is an error, never
a reason to fall back to anything else.
"""
from __future__ import annotations

import ctypes
import pathlib

PKG_DIR = pathlib.Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "_build" / "libgbflow.so"

# status codes (gbflow.h)
GBF_OK, GBF_ERR_ARG, GBF_ERR_CUDA, GBF_ERR_NOMEM, GBF_ERR_NONFINITE, GBF_ERR_UNSTABLE, \
    GBF_ERR_TIMEOUT, GBF_ERR_STATE = range(8)
GBF_SOURCE_DIRICHLET_PATCH, GBF_SOURCE_RATE = 0, 1
GBF_BC_REFERENCE, GBF_BC_HYDROSTATIC_SIDES = 0, 1
GBF_PREC_F64, GBF_PREC_SPLIT, GBF_PREC_SPLIT_DF, GBF_PREC_SPLIT_DEFECT = 0, 1, 2, 3
GBF_OUT_MASS, GBF_OUT_VELOCITY, GBF_OUT_MASS_ARRAYS, GBF_OUT_PROPS, GBF_OUT_CFL = 1, 2, 4, 8, 16

FIELDS = ["P1", "S2", "P2", "ro1", "ro2", "Xi1", "Xi2", "u1x", "u1y", "u1z",
          "u2x", "u2y", "u2z", "roS1", "roS2", "roS1_old", "roS2_old"]
FIELD_ID = {name: i for i, name in enumerate(FIELDS)}
# field order of the gbf_arrays struct (ptr_Arrays order, defines.h:44)
ARRAY_ORDER = ["P1", "P2", "S2", "ro1", "ro2", "u1x", "u1y", "u1z", "u2x", "u2y", "u2z",
               "Xi1", "Xi2", "roS1", "roS1_old", "roS2", "roS2_old"]

_D2 = ctypes.c_double * 2


class GbfModel(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("h1", ctypes.c_double), ("h2", ctypes.c_double), ("h3", ctypes.c_double), ("dt", ctypes.c_double),
        ("K", _D2), ("lam", _D2), ("S_wr", _D2), ("m", _D2), ("P_d", _D2),
        ("beta1", ctypes.c_double), ("beta2", ctypes.c_double),
        ("mu1", ctypes.c_double), ("mu2", ctypes.c_double), ("ro01", ctypes.c_double), ("ro02", ctypes.c_double),
        ("S2_gr", ctypes.c_double), ("P_atm", ctypes.c_double), ("g", ctypes.c_double),
        ("source", ctypes.c_int), ("newton_iterations", ctypes.c_int),
        ("source_mode", ctypes.c_int), ("rate_cells", ctypes.c_int), ("rate", ctypes.c_double),
        ("bc_mode", ctypes.c_int), ("kv", ctypes.c_double), ("newton_tol", ctypes.c_double),
    ]

    @property
    def ncells(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def shape(self):
        """numpy shape (nz, ny, nx) of a C-ordered field with index i + j*nx + k*nx*ny."""
        return (self.nz, self.ny, self.nx)

    def copy(self) -> "GbfModel":
        c = GbfModel()
        ctypes.pointer(c)[0] = self
        return c


class GbfCells(ctypes.Structure):
    _fields_ = [("media", ctypes.POINTER(ctypes.c_int)),
                ("K", ctypes.POINTER(ctypes.c_float)),
                ("phi", ctypes.POINTER(ctypes.c_float))]


class GbfRunDefines(ctypes.Structure):
    _fields_ = [("tau", ctypes.c_double), ("l_w", ctypes.c_double), ("l_n", ctypes.c_double),
                ("c", ctypes.c_double), ("save_plots", ctypes.c_int), ("print_screen", ctypes.c_int)]


class GbfArrays(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in ARRAY_ORDER]


def reference_model(nx: int, ny: int, nz: int, dt: float) -> GbfModel:
    """The reference's constants (defines.h:6-26) and defines.ini defaults.

    Pure Python twin of gbf_model_reference(); the tests check that both agree.
    """
    m = GbfModel()
    m.nx, m.ny, m.nz = nx, ny, nz
    m.h1, m.h2, m.h3, m.dt = 0.02045, 0.01969, 0.01969, dt
    m.K[:] = [6.64e-11, 7.15e-12]
    m.lam[:] = [2.7, 2.0]
    m.S_wr[:] = [0.09, 0.12]
    m.m[:] = [0.4, 0.39]
    m.P_d[:] = [755.0, 2060.0]
    m.beta1, m.beta2 = 1.0e-4, 1.0e-8
    m.mu1, m.mu2, m.ro01, m.ro02 = 0.001, 0.0009, 1000.0, 1460.0
    m.S2_gr, m.P_atm, m.g = 0.4, 100000.0, 9.8
    m.source, m.newton_iterations = 3, 7
    m.source_mode, m.rate_cells, m.rate = GBF_SOURCE_DIRICHLET_PATCH, 0, 0.0
    m.bc_mode, m.kv, m.newton_tol = GBF_BC_REFERENCE, 1.0, 0.0
    return m


_lib = None


def load_library(required: bool = True):
    """Load the in-tree libgbflow.so (built by build.py)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        if required:
            raise RuntimeError(f"libgbflow.so is not built ({LIB_PATH}); run __graft_entry__.build()")
        return None
    lib = ctypes.CDLL(str(LIB_PATH))
    _declare(lib)
    _lib = lib
    return lib


def _declare(lib) -> None:
    c_int, c_double, c_void_p, c_size_t = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_size_t
    PM = ctypes.POINTER(GbfModel)
    PC = ctypes.POINTER(GbfCells)
    sig = {
        "gbf_last_status": (c_int, []),
        "gbf_clear_status": (None, []),
        "gbf_status_string": (ctypes.c_char_p, [c_int]),
        "gbf_version": (ctypes.c_char_p, []),
        "gbf_model_reference": (None, [PM, c_int, c_int, c_int, c_double]),
        "gbf_stable_dt": (c_double, [PM, PC, c_double]),
        "gbf_model_validate": (c_int, [PM, PC, c_int]),
        "gbf_props_f64": (c_int, [PM, GbfArrays, GbfCells, c_void_p]),
        "gbf_velocity_f64": (c_int, [PM, GbfArrays, c_void_p]),
        "gbf_mass_f64": (c_int, [PM, GbfArrays, GbfCells, c_void_p]),
        "gbf_newton_f64": (c_int, [PM, GbfArrays, GbfCells, c_void_p]),
        "gbf_boundary_f64": (c_int, [PM, GbfArrays, c_void_p, c_void_p]),
        "gbf_boundary_scratch_doubles": (c_size_t, [PM]),
        "gbf_boundary_f64_noalloc": (c_int, [PM, GbfArrays, c_void_p]),
        "gbf_abi_sizeof": (c_size_t, [c_int]),
        "gbf_domain_create": (c_int, [PM, PC, c_int, ctypes.POINTER(c_void_p)]),
        "gbf_domain_destroy": (c_int, [c_void_p]),
        "gbf_domain_set_outputs": (c_int, [c_void_p, c_int, c_int]),
        "gbf_domain_set_stream": (c_int, [c_void_p, c_void_p]),
        "gbf_domain_upload": (c_int, [c_void_p, c_void_p, c_void_p]),
        "gbf_domain_upload_device": (c_int, [c_void_p, c_void_p, c_void_p]),
        "gbf_domain_step": (c_int, [c_void_p, c_int]),
        "gbf_domain_download": (c_int, [c_void_p, c_int, c_void_p]),
        "gbf_domain_advance_host": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
        "gbf_domain_mass_history": (c_int, [c_void_p, c_void_p, c_int, ctypes.POINTER(c_int)]),
        "gbf_domain_cfl_history": (c_int, [c_void_p, c_void_p, c_int, ctypes.POINTER(c_int)]),
        "gbf_ensemble_cfl_history": (c_int, [c_void_p, c_void_p, c_int, ctypes.POINTER(c_int)]),
        "gbf_domain_status": (c_int, [c_void_p]),
        "gbf_domain_sync": (c_int, [c_void_p]),
        "gbf_domain_steps_done": (ctypes.c_longlong, [c_void_p]),
        "gbf_domain_launches_per_step": (c_int, [c_void_p]),
        "gbf_dropin_set_mode": (c_int, [c_int]),
        "gbf_dropin_get_mode": (c_int, []),
        "gbf_fill_lognormal_K": (c_int, [c_int, c_int, c_int, ctypes.c_uint64, c_double, c_double, c_double,
                                         c_void_p]),
        "gbf_fill_porosity": (c_int, [c_int, c_int, c_int, ctypes.c_uint64, c_double, c_double, c_void_p]),
        "gbf_fill_lognormal_K_device": (c_int, [c_int, c_int, c_int, ctypes.c_uint64, c_double, c_double, c_double,
                                                c_void_p, c_void_p]),
        "gbf_fill_porosity_device": (c_int, [c_int, c_int, c_int, ctypes.c_uint64, c_double, c_double, c_void_p,
                                             c_void_p]),
        "gbf_domain_set_timing": (c_int, [c_void_p, c_int]),
        "gbf_domain_kernel_times": (c_int, [c_void_p, c_void_p, c_void_p, c_int]),
        "gbf_kernel_kinds": (c_int, []),
        "gbf_kernel_name": (ctypes.c_char_p, [c_int]),
        "gbf_set_tma": (c_int, [c_int]),
        "gbf_set_host_direct": (c_int, [c_int]),
        "gbf_diag_bounded_wait": (c_int, [ctypes.c_uint, ctypes.POINTER(c_double)]),
        "gbf_domain_uses_tma": (c_int, [c_void_p]),
        "gbf_ensemble_uses_tma": (c_int, [c_void_p]),
        "gbf_checkpoint_bytes": (c_size_t, [PM]),
        "gbf_checkpoint_write": (c_int, [ctypes.c_char_p, PM, c_int, c_void_p, c_void_p, c_void_p, c_void_p,
                                         c_void_p]),
        "gbf_checkpoint_read": (c_int, [ctypes.c_char_p, PM, ctypes.POINTER(c_int), c_void_p, c_void_p, c_void_p,
                                        c_void_p, c_void_p]),
        "gbf_domain_save": (c_int, [c_void_p, ctypes.c_char_p, c_int]),
        "gbf_domain_restore": (c_int, [c_void_p, ctypes.c_char_p, ctypes.POINTER(c_int)]),
        "gbf_read_defines": (c_int, [ctypes.c_char_p, PM, ctypes.POINTER(GbfRunDefines)]),
        "gbf_write_plots": (c_int, [ctypes.c_char_p, PM, c_double, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p]),
        "gbf_domain_write_plots": (c_int, [c_void_p, ctypes.c_char_p, c_double]),
        "gbf_ensemble_create": (c_int, [c_int, PM, PC, c_int, ctypes.POINTER(c_void_p)]),
        "gbf_ensemble_destroy": (c_int, [c_void_p]),
        "gbf_ensemble_size": (c_int, [c_void_p]),
        "gbf_ensemble_cells": (ctypes.c_longlong, [c_void_p]),
        "gbf_ensemble_interior_cells": (ctypes.c_longlong, [c_void_p]),
        "gbf_ensemble_set_stream": (c_int, [c_void_p, c_void_p]),
        "gbf_ensemble_set_outputs": (c_int, [c_void_p, c_int, c_int]),
        "gbf_ensemble_upload": (c_int, [c_void_p, c_int, c_void_p, c_void_p]),
        "gbf_ensemble_upload_all": (c_int, [c_void_p, c_void_p, c_void_p]),
        "gbf_ensemble_download_all": (c_int, [c_void_p, c_void_p, c_void_p]),
        "gbf_ensemble_advance_host": (c_int, [c_void_p, c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
        "gbf_ensemble_set_pipeline_groups": (c_int, [c_void_p, c_int]),
        "gbf_ensemble_step": (c_int, [c_void_p, c_int]),
        "gbf_ensemble_download": (c_int, [c_void_p, c_int, c_int, c_void_p]),
        "gbf_ensemble_mass_history": (c_int, [c_void_p, c_void_p, c_int, ctypes.POINTER(c_int)]),
        "gbf_ensemble_status": (c_int, [c_void_p]),
        "gbf_ensemble_sync": (c_int, [c_void_p]),
        "gbf_ensemble_set_timing": (c_int, [c_void_p, c_int]),
        "gbf_ensemble_kernel_times": (c_int, [c_void_p, c_void_p, c_void_p, c_int]),
        "gbf_ensemble_launches_per_step": (c_int, [c_void_p]),
        "gbf_ensemble_set_tuning": (c_int, [c_void_p, c_int, c_int, c_int]),
        "gbf_ensemble_get_tuning": (c_int, [c_void_p, ctypes.POINTER(c_int), c_void_p, c_void_p, c_int]),
        "gbf_ensemble_shape_name": (ctypes.c_char_p, [c_int]),
        "gbf_ensemble_autotune": (c_int, [c_void_p, c_int]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args


def check(status: int, what: str = "") -> None:
    if status != GBF_OK:
        lib = load_library()
        raise RuntimeError(f"gbflow error {status} ({lib.gbf_status_string(status).decode()}) {what}")
