"""Helpers of the GPU parity tests: device mirrors of oracle states (torch is
used only for device memory) and the tolerance checks."""
import ctypes

import numpy as np

# Tolerances of the plain FP64 paths against the FP64 oracle: max |dS| and the
# max-norm error of every other field relative to its largest magnitude.
F64_TOL = 1e-12
# Velocities are first differences of P divided by h: they carry the absolute
# rounding of P (~eps * P) over pressure differences that can be small, so
# paths whose P differs from the oracle's in the last bits (log/exp instead of
# pow, FMA contraction) agree with it to this tolerance.
F64_TOL_GRADIENT = 1e-10


def p_tol(model) -> float:
    """Tolerance on P (max-norm, relative). P is recovered from the phase masses
    through the densities' slope rho0*beta: a relative rounding eps of a mass
    becomes a relative pressure error of about eps / (beta * P). With
    beta = 1e-9 and P ~ 1e5 that condition number is 1e4, so the bound is
    4e-15 times it, and never below 1e-12."""
    cond = 1.0 / (min(model.beta1, model.beta2) * model.P_atm)
    return max(F64_TOL, 4e-15 * cond)


def mass_order_rtol(form: str, wide: float) -> float:
    """Tolerance between phase-mass sums of one state taken in different orders
    (other tilings, single domain vs ensemble). The other split forms sum phi T
    or phi D in FP32 pairs; the FP32 defect form sums phi D in FP32, so its sums move
    by about 2^-24 |sum phi D| / |mass| (D / M up to 1e-5 at compressibility
    1e-4: about 1e-12)."""
    return 2e-11 if form == "split_defect" else wide


def torch():
    import torch as t
    return t


class DevState:
    """Device copies (torch, float64) of every reference array of a State."""

    def __init__(self, st, abi):
        t = torch()
        self.abi = abi
        self.st = st
        self.t = {k: t.as_tensor(np.ascontiguousarray(st[k])).cuda() for k in st.f}
        self.media = t.as_tensor(np.ascontiguousarray(st.media)).cuda()
        self.K = t.as_tensor(st.K).cuda() if st.K is not None else None
        self.phi = t.as_tensor(st.phi).cuda() if st.phi is not None else None

    def arrays(self):
        a = self.abi.GbfArrays()
        for k, v in self.t.items():
            setattr(a, k, v.data_ptr())
        return a

    def cells(self):
        c = self.abi.GbfCells()
        c.media = ctypes.cast(self.media.data_ptr(), ctypes.POINTER(ctypes.c_int))
        c.K = ctypes.cast(self.K.data_ptr(), ctypes.POINTER(ctypes.c_float)) if self.K is not None else None
        c.phi = ctypes.cast(self.phi.data_ptr(), ctypes.POINTER(ctypes.c_float)) if self.phi is not None else None
        return c

    def host(self, k):
        torch().cuda.synchronize()
        return self.t[k].cpu().numpy()


def rel_err(got, want):
    scale = max(float(np.abs(want).max()), 1e-300)
    return float(np.abs(got - want).max()) / scale


def assert_field(name, got, want, tol=F64_TOL):
    assert np.all(np.isfinite(got)), f"{name}: non-finite values"
    if name == "S2":
        err = float(np.abs(got - want).max())
    else:
        err = rel_err(got, want)
    assert err <= tol, f"{name}: error {err:.3e} > {tol:.1e}"
    return err


def rel_l2(got, want):
    return float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300))
