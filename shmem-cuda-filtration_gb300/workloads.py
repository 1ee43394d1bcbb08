"""Synthetic workloads with the shapes, fields and parameters of the benchmark
configurations (seeded; no dataset exists for this simulator).

Common physics of the configurations: water rho0 = 1000 kg/m^3, mu = 1e-3 Pa s;
DNAPL rho0 = 1460 kg/m^3, mu = 9e-4 Pa s; both compressibilities 1e-9 1/Pa;
Brooks-Corey lambda = 2.7, entry pressure 755 Pa, S_wr = 0.1; mass-rate DNAPL
injection into the top-centre cells; hydrostatic Dirichlet P on the sides and
a no-flow bottom; initial state fully water-saturated and hydrostatic (1e5 Pa
at the top).

`lib` is any library that exports the input functions gbf_fill_lognormal_K,
gbf_fill_porosity and gbf_stable_dt: libgbflow, or the same source built
alone for CPU-only callers (they give the same bits).

The time steps quoted with the configurations (0.02-0.05 s) are far above
the explicit scheme's stability bound at compressibility 1e-9 (about 5e-7 s
at 40^3 in a 1 m cube; the reference CPU path diverges within two steps at
0.05 s). Every workload therefore runs at dt = 0.5 x gbf_stable_dt, which is
reported; the metric (cell-steps/s) does not depend on dt.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import abi


@dataclass
class Member:
    model: abi.GbfModel
    K: np.ndarray | None = None
    phi: np.ndarray | None = None
    media: np.ndarray | None = None
    info: dict = field(default_factory=dict)

    @property
    def ncells(self) -> int:
        return self.model.ncells

    def initial_state(self):
        """Hydrostatic pressure (main.cpp:114) and the initial saturation."""
        m = self.model
        j = np.arange(m.ny, dtype=np.float64)[None, :, None]
        P = np.broadcast_to(m.P_atm + j * m.ro01 * m.g * m.h2, m.shape).copy()
        S = np.zeros(m.shape, np.float64)
        if m.source_mode == abi.GBF_SOURCE_DIRICHLET_PATCH:
            i = np.arange(m.nx)
            k = np.arange(m.nz)
            pi = (i >= m.nx // 2 - m.source) & (i <= m.nx // 2 + m.source)
            pk = (k >= m.nz // 2 - m.source) & (k <= m.nz // 2 + m.source)
            S[:, 0, :] = np.where(pk[:, None] & pi[None, :], m.S2_gr, 0.0)
        return P, S


def base_model(n: tuple[int, int, int], length: float, rate: float, rate_cells: int,
               lam: float = 2.7, P_d: float = 755.0, kv: float = 1.0) -> abi.GbfModel:
    nx, ny, nz = n
    m = abi.reference_model(nx, ny, nz, 1.0)
    m.h1, m.h2, m.h3 = length / nx, length / ny, length / nz
    m.beta1 = m.beta2 = 1e-9
    m.S_wr[:] = [0.1, 0.1]
    m.lam[:] = [lam, lam]
    m.P_d[:] = [P_d, P_d]
    m.K[:] = [6.64e-11, 6.64e-11]
    m.m[:] = [0.4, 0.4]
    m.source_mode, m.rate_cells, m.rate = abi.GBF_SOURCE_RATE, rate_cells, rate
    m.bc_mode = abi.GBF_BC_HYDROSTATIC_SIDES
    m.kv = kv
    m.newton_tol = 1e-11
    return m


def set_stable_dt(lib, mem: Member, safety: float = 0.5) -> Member:
    cells = abi.GbfCells()
    if mem.K is not None:
        cells.K = mem.K.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    if mem.phi is not None:
        cells.phi = mem.phi.ctypes.data_as(ctypes.POINTER(ctypes.c_float))
    mem.model.dt = lib.gbf_stable_dt(ctypes.byref(mem.model), ctypes.byref(cells), safety)
    return mem


def fields(lib, shape, seed: int, sigma_lnK: float, corr: float = 8.0):
    nz, ny, nx = shape
    K = np.empty(shape, np.float32)
    phi = np.empty(shape, np.float32)
    for status, what in ((lib.gbf_fill_lognormal_K(nx, ny, nz, seed, 6.64e-11, sigma_lnK, corr, K.ctypes.data),
                          "K field"),
                         (lib.gbf_fill_porosity(nx, ny, nz, seed + 1, 0.35, 0.05, phi.ctypes.data), "porosity")):
        if status != abi.GBF_OK:
            raise RuntimeError(f"{what}: generator status {status}")
    return K, phi


def config0(lib) -> Member:
    """40^3, 1 m cube, homogeneous phi = 0.4, K = 6.64e-11; 1e-4 kg/s into the
    top-centre 3x3 cells; 200 steps."""
    m = base_model((40, 40, 40), 1.0, 1e-4, 3)
    return set_stable_dt(lib, Member(m, info={"config": 0, "steps": 200}))


def config1(lib, n: int = 256, seed: int = 1000) -> Member:
    """256^3, 10 m cube, log-normal K (sigma_lnK = 1, 8-cell Gaussian
    correlation), phi = 0.35 + 0.05 U(-1, 1); 5e-3 kg/s over the top-centre
    8x8 cells; 1000 steps. `n` shrinks the grid for profiling."""
    m = base_model((n, n, n), 10.0, 5e-3, 8)
    K, phi = fields(lib, m.shape, seed, 1.0)
    return set_stable_dt(lib, Member(m, K, phi, info={"config": 1, "steps": 1000, "seed": seed}))


def config1_dropin(lib, n: int = 256) -> Member:
    """Config 1's grid (a 10 m cube of 256^3 cells, compressibility 1e-9) in
    the form the reference's host function set expresses: its 2-entry media
    table (all cells media 0: K = 6.64e-11, phi = 0.4, Brooks-Corey lambda =
    2.7, entry pressure 755 Pa), its Dirichlet saturation patch (S2_gr = 0.4
    over the top-centre 7x7 cells) and boundary rules, and 7 Newton
    iterations. The defines.h calls carry no per-cell field and no rate source."""
    m = abi.reference_model(n, n, n, 1.0)
    m.h1 = m.h2 = m.h3 = 10.0 / n
    m.beta1 = m.beta2 = 1e-9
    return set_stable_dt(lib, Member(m, media=np.zeros(m.shape, np.int32), info={"config": 1, "steps": 1000}))


def config2(lib, seed: int = 2000) -> Member:
    """512x512x256, sigma_lnK = 1.5, same fluids and injection as config 1; 500 steps."""
    m = base_model((512, 512, 256), 10.0, 5e-3, 8)
    m.h3 = 5.0 / 256  # keep cubic cells: the third axis is half as long
    K, phi = fields(lib, m.shape, seed, 1.5)
    return set_stable_dt(lib, Member(m, K, phi, info={"config": 2, "steps": 500, "seed": seed}))


def config3_specs(members: int = 96, seed: int = 3000) -> list[dict]:
    """Parameters of the config-3 realizations, drawn in member order (cheap:
    no fields): cube edges uniform in {64, 96, 128, 160} (cell size 1/32 m),
    sigma_lnK uniform in [0.5, 2], rate uniform in [1e-4, 1e-2] kg/s over the
    top-centre 4x4 cells. Member r's fields come from seed + 1000 (r + 1), so a
    longer list extends a shorter one."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(members):
        e = int(rng.choice([64, 96, 128, 160]))
        sig = float(rng.uniform(0.5, 2.0))
        rate = float(rng.uniform(1e-4, 1e-2))
        out.append({"config": 3, "index": r, "edge": e, "sigma_lnK": sig, "rate": rate,
                    "seed": seed + 1000 * (r + 1)})
    return out


def config4_specs(members: int = 256, seed: int = 4000) -> list[dict]:
    """Parameters of the config-4 realizations, drawn in member order (cheap):
    edges uniform in [48, 128] (multiples of 16), anisotropy kz/kx uniform in
    [0.1, 1] (applied on the vertical axis), entry pressure uniform in
    [500, 1500] Pa, lambda uniform in [2, 3.5], sigma_lnK uniform in [0.5, 2],
    rate uniform in [1e-4, 1e-2] kg/s."""
    rng = np.random.default_rng(seed)
    out = []
    for r in range(members):
        e = int(rng.choice(np.arange(48, 129, 16)))
        kv = float(rng.uniform(0.1, 1.0))
        pd = float(rng.uniform(500.0, 1500.0))
        lam = float(rng.uniform(2.0, 3.5))
        sig = float(rng.uniform(0.5, 2.0))
        rate = float(rng.uniform(1e-4, 1e-2))
        out.append({"config": 4, "index": r, "edge": e, "kv": kv, "P_d": pd, "lambda": lam, "sigma_lnK": sig,
                    "rate": rate, "seed": seed + 1000 * (r + 1)})
    return out


def spec_cells(spec: dict) -> int:
    return spec["edge"] ** 3


def build_member(lib, spec: dict) -> Member:
    """One realization of a spec: its grid, seeded fields and stable dt."""
    e = spec["edge"]
    if spec["config"] == 3:
        m = base_model((e, e, e), e / 32.0, spec["rate"], 4)
    else:
        m = base_model((e, e, e), e / 32.0, spec["rate"], 4, lam=spec["lambda"], P_d=spec["P_d"], kv=spec["kv"])
    K, phi = fields(lib, m.shape, spec["seed"], spec["sigma_lnK"])
    info = {k: v for k, v in spec.items() if k not in ("config", "seed")}
    return set_stable_dt(lib, Member(m, K, phi, info=info))


def shard(items: list, rank: int, world: int) -> list:
    """The share of rank `rank` of `world` ranks: items rank, rank + world, ...
    Every item belongs to exactly one rank; one rank takes them all."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError(f"rank {rank} of {world}")
    return items[rank::world]


def config3(lib, members: int = 96, seed: int = 3000) -> list[Member]:
    """96 realizations, cube edges uniform in {64, 96, 128, 160}; 500 steps."""
    return [build_member(lib, s) for s in config3_specs(members, seed)]


def config4(lib, members: int = 256, seed: int = 4000) -> list[Member]:
    """256 realizations, edges uniform in [48, 128] (multiples of 16),
    anisotropic, with per-member closures; 1000 steps."""
    return [build_member(lib, s) for s in config4_specs(members, seed)]
