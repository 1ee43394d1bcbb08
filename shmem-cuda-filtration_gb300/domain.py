"""Python wrapper of the gbf_domain C ABI (include/gbflow.h)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi


def cells_struct(media=None, K=None, phi=None):
    """A GbfCells over host numpy arrays (kept alive by the caller)."""
    c = abi.GbfCells()
    c.media = media.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if media is not None else None
    c.K = K.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if K is not None else None
    c.phi = phi.ctypes.data_as(ctypes.POINTER(ctypes.c_float)) if phi is not None else None
    return c


class Domain:
    """One grid on the GPU; state stays in HBM between steps."""

    def __init__(self, model, media=None, K=None, phi=None, precision=abi.GBF_PREC_F64):
        self.lib = abi.load_library()
        self.model = model.copy()
        self._media = None if media is None else np.ascontiguousarray(media, np.int32)
        self._K = None if K is None else np.ascontiguousarray(K, np.float32)
        self._phi = None if phi is None else np.ascontiguousarray(phi, np.float32)
        cells = cells_struct(self._media, self._K, self._phi)
        h = ctypes.c_void_p()
        abi.check(self.lib.gbf_domain_create(ctypes.byref(self.model), ctypes.byref(cells), precision, ctypes.byref(h)),
                  "gbf_domain_create")
        self.h = h
        self.precision = precision

    def close(self):
        if self.h:
            self.lib.gbf_domain_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_outputs(self, flags: int, mass_history: int = 0):
        abi.check(self.lib.gbf_domain_set_outputs(self.h, flags, mass_history), "set_outputs")

    def set_stream(self, stream_ptr: int):
        abi.check(self.lib.gbf_domain_set_stream(self.h, ctypes.c_void_p(stream_ptr)), "set_stream")

    def upload(self, P1: np.ndarray, S2: np.ndarray):
        P1 = np.ascontiguousarray(P1, np.float64)
        S2 = np.ascontiguousarray(S2, np.float64)
        assert P1.size == self.model.ncells and S2.size == self.model.ncells
        abi.check(self.lib.gbf_domain_upload(self.h, P1.ctypes.data, S2.ctypes.data), "upload")
        self.sync()

    def upload_device(self, P1_ptr: int, S2_ptr: int):
        abi.check(self.lib.gbf_domain_upload_device(self.h, P1_ptr, S2_ptr), "upload_device")

    def step(self, n: int = 1):
        abi.check(self.lib.gbf_domain_step(self.h, n), "step")

    def sync(self):
        abi.check(self.lib.gbf_domain_sync(self.h), "sync")

    def status(self) -> int:
        return self.lib.gbf_domain_status(self.h)

    def advance_host(self, P_in: np.ndarray, S_in: np.ndarray, nsteps: int,
                     P_out: np.ndarray | None = None, S_out: np.ndarray | None = None):
        """upload + nsteps steps + download of P1 and S2 in one call, pipelined
        over slabs of planes for one split-form step (outputs default to the
        inputs, updated in place)."""
        P_out = P_in if P_out is None else P_out
        S_out = S_in if S_out is None else S_out
        for a in (P_in, S_in, P_out, S_out):
            assert a.dtype == np.float64 and a.size == self.model.nx * self.model.ny * self.model.nz
            assert a.flags.c_contiguous
        abi.check(self.lib.gbf_domain_advance_host(self.h, P_in.ctypes.data, S_in.ctypes.data, nsteps,
                                                   P_out.ctypes.data, S_out.ctypes.data), "advance_host")

    def download(self, field: str, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.model.shape, np.float64)
        abi.check(self.lib.gbf_domain_download(self.h, abi.FIELD_ID[field], out.ctypes.data), f"download {field}")
        return out

    def save(self, path, step: int):
        """Checkpoint in the reference's save/save.dat layout."""
        abi.check(self.lib.gbf_domain_save(self.h, str(path).encode(), step), "save")

    def restore(self, path) -> int:
        """Upload (P1, S2) from such a checkpoint; returns its step."""
        j = ctypes.c_int()
        abi.check(self.lib.gbf_domain_restore(self.h, str(path).encode(), ctypes.byref(j)), "restore")
        return j.value

    def write_plots(self, directory, t: float):
        """The reference's Tecplot files (save_data_plots) under `directory`."""
        abi.check(self.lib.gbf_domain_write_plots(self.h, str(directory).encode(), t), "write_plots")

    def cfl_history(self, max_steps: int) -> np.ndarray:
        """CFL numbers [step][2] (GBF_OUT_CFL with GBF_OUT_MASS)."""
        out = np.zeros((max_steps, 2), np.float32)
        n = ctypes.c_int()
        abi.check(self.lib.gbf_domain_cfl_history(self.h, out.ctypes.data, max_steps, ctypes.byref(n)), "cfl")
        return out[: n.value]

    def mass_history(self, max_steps: int) -> np.ndarray:
        out = np.zeros((max_steps, 2), np.float64)
        n = ctypes.c_int()
        abi.check(self.lib.gbf_domain_mass_history(self.h, out.ctypes.data, max_steps, ctypes.byref(n)), "mass")
        return out[: n.value]

    @property
    def launches_per_step(self) -> int:
        return self.lib.gbf_domain_launches_per_step(self.h)

    def set_timing(self, on: bool):
        abi.check(self.lib.gbf_domain_set_timing(self.h, int(on)), "set_timing")

    def kernel_times(self) -> dict:
        """{kernel name: (total ms, launches)} since the last call."""
        n = self.lib.gbf_kernel_kinds()
        ms = np.zeros(n, np.float64)
        cnt = np.zeros(n, np.int32)
        abi.check(self.lib.gbf_domain_kernel_times(self.h, ms.ctypes.data, cnt.ctypes.data, n), "kernel_times")
        return {self.lib.gbf_kernel_name(k).decode(): (float(ms[k]), int(cnt[k])) for k in range(n) if cnt[k]}
