"""Python bindings of the oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module; it is the checker and never the thing measured or shipped.

Three libraries are wrapped:
  * _build/libgbf_oracle.so — the C restatement (gbf_oracle.c), always built;
  * _build/libgbf_inputs.so — the product's seeded field generator and
    stability bound (gbf_fields.cpp) built alone, so that the timed reference
    CPU run makes the same inputs without loading libgbflow;
  * _ref/libgbf_refcpu.so   — the reference's own cpu.cpp/main.cpp/
    no_communication.cpp compiled from their sources (only where the
    reference sources exist at build time).
"""
from __future__ import annotations

import ctypes
import pathlib
import subprocess

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ORACLE_SO = HERE / "_build" / "libgbf_oracle.so"
REF_SO = HERE / "_ref" / "libgbf_refcpu.so"
INPUTS_SO = HERE / "_build" / "libgbf_inputs.so"

# Field order of the reference's ptr_Arrays after x, y, z (defines.h:44).
ARRAY_ORDER = ["P1", "P2", "S2", "ro1", "ro2", "u1x", "u1y", "u1z", "u2x", "u2y", "u2z",
               "Xi1", "Xi2", "roS1", "roS1_old", "roS2", "roS2_old"]


def build() -> None:
    """Compile the oracle (and the reference library when its sources exist)."""
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)


_inputs = None


def inputs_library(abi):
    """libgbf_inputs.so with the signatures of gbf_fill_lognormal_K,
    gbf_fill_porosity and gbf_stable_dt (the same C symbols and results as
    libgbflow's)."""
    global _inputs
    if _inputs is None:
        if not INPUTS_SO.exists():
            build()
        lib = ctypes.CDLL(str(INPUTS_SO))
        c_int, c_double, c_void_p = ctypes.c_int, ctypes.c_double, ctypes.c_void_p
        lib.gbf_fill_lognormal_K.restype = c_int
        lib.gbf_fill_lognormal_K.argtypes = [c_int, c_int, c_int, ctypes.c_uint64, c_double, c_double, c_double,
                                             c_void_p]
        lib.gbf_fill_porosity.restype = c_int
        lib.gbf_fill_porosity.argtypes = [c_int, c_int, c_int, ctypes.c_uint64, c_double, c_double, c_void_p]
        lib.gbf_stable_dt.restype = c_double
        lib.gbf_stable_dt.argtypes = [ctypes.POINTER(abi.GbfModel), ctypes.POINTER(abi.GbfCells), c_double]
        _inputs = lib
    return _inputs


class Consts(ctypes.Structure):
    """Mirror of the reference's `consts` (defines.h:50-61)."""
    _fields_ = [("K", ctypes.c_double * 2), ("lam", ctypes.c_double * 2), ("S_wr", ctypes.c_double * 2),
                ("m", ctypes.c_double * 2), ("P_d", ctypes.c_double * 2),
                ("h1", ctypes.c_double), ("h2", ctypes.c_double), ("h3", ctypes.c_double),
                ("dt", ctypes.c_double), ("tau", ctypes.c_double), ("l_w", ctypes.c_double),
                ("l_n", ctypes.c_double), ("c", ctypes.c_double), ("beta1", ctypes.c_double),
                ("beta2", ctypes.c_double),
                ("NX", ctypes.c_int), ("Ny", ctypes.c_int), ("Nz", ctypes.c_int),
                ("source", ctypes.c_int), ("save_plots", ctypes.c_int), ("print_screen", ctypes.c_int)]


def consts_from_model(m) -> Consts:
    """The reference `consts` equivalent of a reference-mode gbf_model."""
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


class State:
    """All reference arrays of one grid as C-ordered float64 numpy arrays of
    shape (nz, ny, nx); index i + j*nx + k*nx*ny as in the reference."""

    def __init__(self, model, media=None, K=None, phi=None):
        shape = (model.nz, model.ny, model.nx)
        self.model = model
        self.f = {n: np.zeros(shape, np.float64) for n in ARRAY_ORDER}
        self.xyz = [np.zeros(shape, np.float64) for _ in range(3)]
        self.media = np.zeros(shape, np.int32) if media is None else np.ascontiguousarray(media, np.int32)
        self.K = None if K is None else np.ascontiguousarray(K, np.float32)
        self.phi = None if phi is None else np.ascontiguousarray(phi, np.float32)

    def __getitem__(self, k):
        return self.f[k]

    def copy(self) -> "State":
        s = State(self.model, self.media.copy(), None if self.K is None else self.K.copy(),
                  None if self.phi is None else self.phi.copy())
        for n in ARRAY_ORDER:
            s.f[n][...] = self.f[n]
        return s

    def _ptr(self, a):
        return a.ctypes.data_as(ctypes.c_void_p)

    def gbf_arrays(self, abi):
        arr = abi.GbfArrays()
        for n in ARRAY_ORDER:
            setattr(arr, n, self.f[n].ctypes.data)
        return arr

    def gbf_cells(self, abi):
        c = abi.GbfCells()
        c.media = self.media.ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        c.K = self.K.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if self.K is not None else None
        c.phi = self.phi.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if self.phi is not None else None
        return c

    def ref_pointers(self):
        ptrs = (ctypes.c_void_p * 20)()
        for i, a in enumerate(self.xyz):
            ptrs[i] = a.ctypes.data
        for i, n in enumerate(ARRAY_ORDER):
            ptrs[3 + i] = self.f[n].ctypes.data
        return ptrs


class Oracle:
    """The C restatement (gbf_oracle.c)."""

    def __init__(self, abi):
        if not ORACLE_SO.exists():
            build()
        self.abi = abi
        lib = ctypes.CDLL(str(ORACLE_SO))
        PM, PC = ctypes.POINTER(abi.GbfModel), ctypes.POINTER(abi.GbfCells)
        for name in ("orc_props", "orc_mass", "orc_newton"):
            getattr(lib, name).argtypes = [PM, PC, abi.GbfArrays]
        for name in ("orc_velocity", "orc_boundary", "orc_initial"):
            getattr(lib, name).argtypes = [PM, abi.GbfArrays]
        lib.orc_step.argtypes = [PM, PC, abi.GbfArrays, ctypes.c_int, ctypes.c_void_p]
        lib.orc_mass_totals.argtypes = [PM, PC, abi.GbfArrays, ctypes.c_void_p]
        lib.orc_in_rate_patch.argtypes = [PM, ctypes.c_int, ctypes.c_int]
        lib.orc_set_fp32_mobilities.argtypes = [ctypes.c_int]
        self.lib = lib

    def fp32_mobilities(self, level):
        """Experiment switch: round the flux stage's upwinded mobilities to
        FP32, everything else FP64 (False / 0: the bit-exact reference; True /
        1: every face; 2: every face but the DNAPL faces between the
        Dirichlet patch and the cells below it)."""
        self.lib.orc_set_fp32_mobilities(int(level))

    def _call(self, name, st: State, with_cells=True):
        m = ctypes.byref(st.model)
        fn = getattr(self.lib, name)
        if with_cells:
            cells = st.gbf_cells(self.abi)
            fn(m, ctypes.byref(cells), st.gbf_arrays(self.abi))
        else:
            fn(m, st.gbf_arrays(self.abi))

    def initial(self, st: State):
        self._call("orc_initial", st, with_cells=False)

    def props(self, st):
        self._call("orc_props", st)

    def velocity(self, st):
        self._call("orc_velocity", st, with_cells=False)

    def mass(self, st):
        self._call("orc_mass", st)

    def newton(self, st):
        self._call("orc_newton", st)

    def boundary(self, st):
        self._call("orc_boundary", st, with_cells=False)

    def step(self, st: State, nsteps: int = 1, want_mass: bool = False):
        mass = np.zeros((nsteps, 2), np.float64) if want_mass else None
        cells = st.gbf_cells(self.abi)
        self.lib.orc_step(ctypes.byref(st.model), ctypes.byref(cells), st.gbf_arrays(self.abi), nsteps,
                          mass.ctypes.data if mass is not None else None)
        return mass

    def mass_totals(self, st: State):
        out = np.zeros(2, np.float64)
        cells = st.gbf_cells(self.abi)
        self.lib.orc_mass_totals(ctypes.byref(st.model), ctypes.byref(cells), st.gbf_arrays(self.abi),
                                 out.ctypes.data)
        return out


class Reference:
    """The reference's own CPU backend (cpu.cpp + main.cpp + no_communication.cpp),
    compiled from its sources into _ref/. Reference mode only (media table)."""

    @staticmethod
    def available() -> bool:
        return REF_SO.exists()

    def __init__(self):
        lib = ctypes.CDLL(str(REF_SO))
        PP, PI, PCo = ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Consts)
        lib.ref_sizeof_consts.restype = ctypes.c_int
        assert lib.ref_sizeof_consts() == ctypes.sizeof(Consts), "consts layout mismatch"
        lib.ref_initial_data.argtypes = [PP, PI, PCo]
        lib.ref_time_steps.argtypes = [PP, PI, PCo, ctypes.c_int]
        for name in ("ref_ro_P2_Xi", "ref_u", "ref_P1_S2", "ref_boundary"):
            getattr(lib, name).argtypes = [PP, PI, PCo]
        lib.ref_roS.argtypes = [PP, PI, PCo, ctypes.c_double]
        lib.ref_save.argtypes = [ctypes.c_char_p, PP, PI, PCo, ctypes.c_int]
        lib.ref_restore.argtypes = [ctypes.c_char_p, PP, PI, PCo, ctypes.POINTER(ctypes.c_int)]
        lib.ref_plots.argtypes = [ctypes.c_char_p, PP, PI, PCo, ctypes.c_double]
        self.lib = lib

    def _args(self, st):
        return st.ref_pointers(), st.media.ctypes.data, ctypes.byref(consts_from_model(st.model))

    def initial(self, st):
        p, md, c = self._args(st)
        self.lib.ref_initial_data(p, md, c)

    def step(self, st, nsteps=1):
        p, md, c = self._args(st)
        self.lib.ref_time_steps(p, md, c, nsteps)

    def props(self, st):
        self.lib.ref_ro_P2_Xi(*self._args(st))

    def velocity(self, st):
        self.lib.ref_u(*self._args(st))

    def mass(self, st, t=1.0):
        p, md, c = self._args(st)
        self.lib.ref_roS(p, md, c, t)

    def newton(self, st):
        self.lib.ref_P1_S2(*self._args(st))

    def boundary(self, st):
        self.lib.ref_boundary(*self._args(st))

    def save(self, st, directory, j):
        """main.cpp:485 save() into `directory`/save/save.dat."""
        p, md, c = self._args(st)
        assert self.lib.ref_save(str(directory).encode(), p, md, c, j) == 0

    def plots(self, st, directory, t):
        """main.cpp:319 save_data_plots() writing into `directory`."""
        p, md, c = self._args(st)
        assert self.lib.ref_plots(str(directory).encode(), p, md, c, t) == 0

    def restore(self, st, directory) -> int:
        """main.cpp:541 restore() from `directory`/save/save.dat; returns the step."""
        p, md, c = self._args(st)
        j = ctypes.c_int(0)
        assert self.lib.ref_restore(str(directory).encode(), p, md, c, ctypes.byref(j)) == 0
        return j.value
