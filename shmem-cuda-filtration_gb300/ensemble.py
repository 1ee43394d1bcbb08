"""Python wrapper of the gbf_ensemble C ABI (include/gbflow.h)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import abi


class Ensemble:
    """Independent realizations advanced together on the GPU."""

    def __init__(self, members, precision=abi.GBF_PREC_SPLIT_DF):
        """`members`: objects with .model (GbfModel) and optional .media/.K/.phi arrays."""
        self.lib = abi.load_library()
        self.members = members
        n = len(members)
        self._models = (abi.GbfModel * n)()
        self._cells = (abi.GbfCells * n)()
        self._keep = []
        for r, mem in enumerate(members):
            self._models[r] = mem.model
            media = getattr(mem, "media", None)
            K = getattr(mem, "K", None)
            phi = getattr(mem, "phi", None)
            for arr, name, ct in ((media, "media", ctypes.c_int), (K, "K", ctypes.c_float),
                                  (phi, "phi", ctypes.c_float)):
                if arr is not None:
                    arr = np.ascontiguousarray(arr, np.int32 if name == "media" else np.float32)
                    self._keep.append(arr)
                    setattr(self._cells[r], name, arr.ctypes.data_as(ctypes.POINTER(ct)))
        h = ctypes.c_void_p()
        abi.check(self.lib.gbf_ensemble_create(n, self._models, self._cells, precision, ctypes.byref(h)),
                  "gbf_ensemble_create")
        self.h = h
        self.n = n
        self.precision = precision

    def close(self):
        if self.h:
            self.lib.gbf_ensemble_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def cells(self) -> int:
        return self.lib.gbf_ensemble_cells(self.h)

    @property
    def interior_cells(self) -> int:
        return self.lib.gbf_ensemble_interior_cells(self.h)

    def set_outputs(self, flags: int, mass_history: int = 0):
        abi.check(self.lib.gbf_ensemble_set_outputs(self.h, flags, mass_history), "set_outputs")

    def set_stream(self, stream_ptr: int):
        abi.check(self.lib.gbf_ensemble_set_stream(self.h, ctypes.c_void_p(stream_ptr)), "set_stream")

    def upload(self, r: int, P: np.ndarray, S: np.ndarray):
        P = np.ascontiguousarray(P, np.float64)
        S = np.ascontiguousarray(S, np.float64)
        abi.check(self.lib.gbf_ensemble_upload(self.h, r, P.ctypes.data, S.ctypes.data), f"upload {r}")

    def upload_initial(self):
        for r, mem in enumerate(self.members):
            P, S = mem.initial_state()
            self.upload(r, P, S)
        self.sync()

    def offsets(self):
        """Start of each member in the packed all-members layout."""
        return np.concatenate([[0], np.cumsum([m.model.ncells for m in self.members])])

    def upload_all(self, P_all: np.ndarray, S_all: np.ndarray):
        assert P_all.dtype == np.float64 and S_all.dtype == np.float64
        assert P_all.size == self.cells and S_all.size == self.cells
        abi.check(self.lib.gbf_ensemble_upload_all(self.h, P_all.ctypes.data, S_all.ctypes.data), "upload_all")

    def download_all(self, P_all: np.ndarray, S_all: np.ndarray):
        assert P_all.size == self.cells and S_all.size == self.cells
        abi.check(self.lib.gbf_ensemble_download_all(self.h, P_all.ctypes.data, S_all.ctypes.data), "download_all")

    def advance_host(self, P_in: np.ndarray, S_in: np.ndarray, nsteps: int,
                     P_out: np.ndarray | None = None, S_out: np.ndarray | None = None):
        """upload_all + nsteps steps + download_all, pipelined over member
        groups (outputs default to the inputs, updated in place)."""
        P_out = P_in if P_out is None else P_out
        S_out = S_in if S_out is None else S_out
        for a in (P_in, S_in, P_out, S_out):
            assert a.dtype == np.float64 and a.size == self.cells and a.flags.c_contiguous
        abi.check(self.lib.gbf_ensemble_advance_host(self.h, P_in.ctypes.data, S_in.ctypes.data, nsteps,
                                                     P_out.ctypes.data, S_out.ctypes.data), "advance_host")

    def step(self, n: int = 1):
        abi.check(self.lib.gbf_ensemble_step(self.h, n), "step")

    def sync(self):
        abi.check(self.lib.gbf_ensemble_sync(self.h), "sync")

    def status(self) -> int:
        return self.lib.gbf_ensemble_status(self.h)

    def download(self, r: int, field: str, out: np.ndarray | None = None) -> np.ndarray:
        m = self.members[r].model
        if out is None:
            out = np.empty(m.shape, np.float64)
        abi.check(self.lib.gbf_ensemble_download(self.h, r, abi.FIELD_ID[field], out.ctypes.data), "download")
        return out

    def cfl_history(self, max_steps: int) -> np.ndarray:
        """CFL numbers [step][member][2] (GBF_OUT_CFL with GBF_OUT_MASS)."""
        out = np.zeros((max_steps, self.n, 2), np.float32)
        k = ctypes.c_int()
        abi.check(self.lib.gbf_ensemble_cfl_history(self.h, out.ctypes.data, max_steps, ctypes.byref(k)), "cfl")
        return out[: k.value]

    def mass_history(self, max_steps: int) -> np.ndarray:
        out = np.zeros((max_steps, self.n, 2), np.float64)
        k = ctypes.c_int()
        abi.check(self.lib.gbf_ensemble_mass_history(self.h, out.ctypes.data, max_steps, ctypes.byref(k)), "mass")
        return out[: k.value]

    def set_timing(self, on: bool):
        abi.check(self.lib.gbf_ensemble_set_timing(self.h, int(on)), "set_timing")

    def kernel_times(self) -> dict:
        n = self.lib.gbf_kernel_kinds()
        ms = np.zeros(n, np.float64)
        cnt = np.zeros(n, np.int32)
        abi.check(self.lib.gbf_ensemble_kernel_times(self.h, ms.ctypes.data, cnt.ctypes.data, n), "kernel_times")
        return {self.lib.gbf_kernel_name(k).decode(): (float(ms[k]), int(cnt[k])) for k in range(n) if cnt[k]}

    @property
    def launches_per_step(self) -> int:
        return self.lib.gbf_ensemble_launches_per_step(self.h)

    def set_tuning(self, shape: int = -1, edge: int = 0, kchunk: int = 0):
        abi.check(self.lib.gbf_ensemble_set_tuning(self.h, shape, edge, kchunk), "set_tuning")

    def tuning(self) -> dict:
        shape = ctypes.c_int()
        edges = np.zeros(64, np.int32)
        kcs = np.zeros(64, np.int32)
        q = self.lib.gbf_ensemble_get_tuning(self.h, ctypes.byref(shape), edges.ctypes.data, kcs.ctypes.data, 64)
        return {"tile": self.lib.gbf_ensemble_shape_name(shape.value).decode(),
                "kchunk_by_edge": {int(edges[i]): int(kcs[i]) for i in range(q)}}

    def autotune(self, trial_steps: int = 2) -> dict:
        abi.check(self.lib.gbf_ensemble_autotune(self.h, trial_steps), "autotune")
        return self.tuning()
