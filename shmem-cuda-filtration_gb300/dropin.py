"""ctypes bindings of the drop-in: the reference's GPU host function set
(defines.h:63-116) exported by libgbflow.so with C++ linkage.

These call exactly the symbols the reference driver (main.cpp) links to, so a
Python caller exercises the same boundary as the C++ one. The structs mirror
ptr_Arrays (defines.h:41-47) and consts (defines.h:50-61).
"""
from __future__ import annotations

import ctypes

from . import abi

PTR_FIELDS = ["x", "y", "z", "P1", "P2", "S2", "ro1", "ro2", "u1x", "u1y", "u1z", "u2x", "u2y", "u2z",
              "Xi1", "Xi2", "roS1", "roS1_old", "roS2", "roS2_old"]


class PtrArrays(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in PTR_FIELDS] + [("media", ctypes.c_void_p)]


class Consts(ctypes.Structure):
    _fields_ = [("K", ctypes.c_double * 2), ("lam", ctypes.c_double * 2), ("S_wr", ctypes.c_double * 2),
                ("m", ctypes.c_double * 2), ("P_d", ctypes.c_double * 2),
                ("h1", ctypes.c_double), ("h2", ctypes.c_double), ("h3", ctypes.c_double),
                ("dt", ctypes.c_double), ("tau", ctypes.c_double), ("l_w", ctypes.c_double),
                ("l_n", ctypes.c_double), ("c", ctypes.c_double), ("beta1", ctypes.c_double),
                ("beta2", ctypes.c_double),
                ("NX", ctypes.c_int), ("Ny", ctypes.c_int), ("Nz", ctypes.c_int),
                ("source", ctypes.c_int), ("save_plots", ctypes.c_int), ("print_screen", ctypes.c_int)]


def consts_from_model(m) -> Consts:
    c = Consts()
    c.K[:] = list(m.K)
    c.lam[:] = list(m.lam)
    c.S_wr[:] = list(m.S_wr)
    c.m[:] = list(m.m)
    c.P_d[:] = list(m.P_d)
    c.h1, c.h2, c.h3, c.dt = m.h1, m.h2, m.h3, m.dt
    c.tau, c.l_w, c.l_n, c.c = 0.002, 2e-7, 8.528784e-10, 1407.0
    c.beta1, c.beta2 = m.beta1, m.beta2
    c.NX, c.Ny, c.Nz = m.nx, m.ny, m.nz
    c.source, c.save_plots, c.print_screen = m.source, 100000, 1000
    return c


# Mangled names of the defines.h prototypes (Itanium C++ ABI).
SYMBOLS = {
    "ro_P2_Xi_calculation": "_Z20ro_P2_Xi_calculation14ptr_Arrays_tagS_10consts_tagiiiiii",
    "u_calculation": "_Z13u_calculation14ptr_Arrays_tagS_iiiiii10consts_tag",
    "roS_calculation": "_Z15roS_calculation14ptr_Arrays_tagS_10consts_tagdiiiiii",
    "P1_S2_calculation": "_Z17P1_S2_calculation14ptr_Arrays_tagS_10consts_tagiiiiii",
    "boundary_conditions": "_Z19boundary_conditions14ptr_Arrays_tagS_iiiiii10consts_tag",
    "load_data_to_host": "_Z17load_data_to_hostPdS_i10consts_tag",
    "load_data_to_device": "_Z19load_data_to_devicePdS_i10consts_tag",
    "load_data_to_device_int": "_Z23load_data_to_device_intPiS_i10consts_tag",
    "device_memory_alloc": "_Z19device_memory_allocP14ptr_Arrays_tagPPdi10consts_tag",
    "device_memory_free": "_Z18device_memory_free14ptr_Arrays_tagPd",
    "Device_Initialize": "_Z17Device_InitializeiPiS_S_i10consts_tag",
    "load_exchange_data": "_Z18load_exchange_dataPdS_S_S_iiiii10consts_tag",
    "save_exchange_data": "_Z18save_exchange_dataPdS_S_S_iiiii10consts_tag",
}


class DropIn:
    """The reference's host function set, called like main.cpp calls it."""

    def __init__(self):
        lib = abi.load_library()
        self.lib = lib
        i, d, v, PA, C = ctypes.c_int, ctypes.c_double, ctypes.c_void_p, PtrArrays, Consts
        f = {}
        for name, sym in SYMBOLS.items():
            f[name] = getattr(lib, sym)
            f[name].restype = None
        f["ro_P2_Xi_calculation"].argtypes = [PA, PA, C, i, i, i, i, i, i]
        f["u_calculation"].argtypes = [PA, PA, i, i, i, i, i, i, C]
        f["roS_calculation"].argtypes = [PA, PA, C, d, i, i, i, i, i, i]
        f["P1_S2_calculation"].argtypes = [PA, PA, C, i, i, i, i, i, i]
        f["boundary_conditions"].argtypes = [PA, PA, i, i, i, i, i, i, C]
        f["load_data_to_host"].argtypes = [v, v, i, C]
        f["load_data_to_device"].argtypes = [v, v, i, C]
        f["load_data_to_device_int"].argtypes = [v, v, i, C]
        f["device_memory_alloc"].argtypes = [ctypes.POINTER(PA), ctypes.POINTER(v), i, C]
        f["device_memory_free"].argtypes = [PA, v]
        f["Device_Initialize"].argtypes = [i, ctypes.POINTER(i), ctypes.POINTER(i), ctypes.POINTER(i), i, C]
        self.f = f
        lib.gbf_dropin_set_mode.argtypes = [ctypes.c_int]
        lib.gbf_dropin_domain.restype = ctypes.c_void_p
        lib.gbf_dropin_domain.argtypes = [ctypes.c_void_p]

    def domain(self, dev_P1) -> int | None:
        """Handle of the gbflow domain behind fused-mode arrays (gbf_dropin_domain)."""
        return self.lib.gbf_dropin_domain(dev_P1)

    def set_mode(self, mode: int):
        abi.check(self.lib.gbf_dropin_set_mode(mode), "gbf_dropin_set_mode")

    def time_step(self, H: PtrArrays, D: PtrArrays, c: Consts, t: float, bX=0, bY=0, bZ=0):
        """time_step_function (main.cpp:83-94) with the single-domain
        exchanges of no_communication.cpp, which are empty."""
        n = c.NX
        self.f["ro_P2_Xi_calculation"](H, D, c, n, 0, 1, bX, bY, bZ)
        self.f["u_calculation"](H, D, n, 0, 1, bX, bY, bZ, c)
        self.f["roS_calculation"](H, D, c, t, n, 0, 1, bX, bY, bZ)
        self.f["P1_S2_calculation"](H, D, c, n, 0, 1, bX, bY, bZ)
        self.f["boundary_conditions"](H, D, n, 0, 1, bX, bY, bZ, c)
