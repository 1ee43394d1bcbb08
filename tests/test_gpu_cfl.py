"""CFL numbers of the split step (GBF_OUT_CFL): the device's per-step maxima
against an FP64 restatement of their definition on the state each step
starts from, and ensembles against single domains (maxima: bit for bit)."""
import ctypes

import numpy as np
import pytest

from test_gpu_f64 import make_case

pytestmark = pytest.mark.gpu


def cfl_reference(m, P, S, K, phi):
    """max over interior cells and faces of |x L_upwind| / (rho0 h) * dt / phi
    per phase; x = potential gradient of the face (gravity on y faces with the
    centre cell's density, cpu.cpp:257-258; no flow through the bottom face
    with hydrostatic sides), L = -K kr rho / mu (Brooks-Corey, cpu.cpp:60-62),
    densities at P2 = P1."""
    se = (1.0 - S - m.S_wr[0]) / (1.0 - m.S_wr[0])
    kr1 = se ** ((2.0 + 3.0 * m.lam[0]) / m.lam[0])
    kr2 = (1.0 - se) ** 2 * (1.0 - se ** ((2.0 + m.lam[0]) / m.lam[0]))
    ro1 = m.ro01 * (1.0 + m.beta1 * (P - m.P_atm))
    ro2 = m.ro02 * (1.0 + m.beta2 * (P - m.P_atm))
    Ks = K.astype(np.float64)
    L = [-Ks * kr1 * ro1 / m.mu1, -Ks * kr2 * ro2 / m.mu2]
    ro = [ro1, ro2]
    rho0 = [m.ro01, m.ro02]
    c = (slice(1, -1),) * 3
    out = []
    for a in range(2):
        best = np.zeros(P[c].shape)
        # axis 2 = x (i), axis 1 = y (j, gravity), axis 0 = z (k)
        for ax, h, w in ((2, m.h1, 1.0), (1, m.h2, m.kv), (0, m.h3, 1.0)):
            def sh(A, d):
                sl = [slice(1, -1)] * 3
                sl[ax] = slice(1 + d, A.shape[ax] - 1 + d)
                return A[tuple(sl)]
            Pc, Pm, Pp = P[c], sh(P, -1), sh(P, 1)
            Lc, Lm, Lp = L[a][c], sh(L[a], -1), sh(L[a], 1)
            g = ro[a][c] * m.g if ax == 1 else 0.0
            x1 = (Pm - Pc) / h + g  # into the cell from the minus side
            x2 = (Pc - Pp) / h + g  # out through the plus side
            if ax == 1 and m.bc_mode == 1:  # GBF_BC_HYDROSTATIC_SIDES: no-flow bottom face
                x2 = x2.copy()
                x2[:, -1, :] = 0.0
            f1 = np.abs(x1 * np.where(x1 >= 0, Lm, Lc))
            f2 = np.abs(x2 * np.where(x2 >= 0, Lc, Lp))
            best = np.maximum(best, w * np.maximum(f1, f2) / h)
        out.append(float((best * m.dt / phi[c].astype(np.float64) / rho0[a]).max()))
    return out


@pytest.mark.parametrize("form", ["split", "split_df", "split_defect"])
def test_cfl_matches_definition(gpu_lib, abi, O, oracle, pkg, form):
    from importlib import import_module
    Domain = import_module(pkg.__name__ + ".domain").Domain
    m, st, _ = make_case(abi, O, gpu_lib, "heterogeneous_aniso_24x20x18")
    m.S_wr[:] = [0.1, 0.1]
    oracle.initial(st)
    st["S2"][3:12, 2:9, 6:16] = 0.3  # a DNAPL blob, so that both phases are mobile
    p = {"split": abi.GBF_PREC_SPLIT, "split_df": abi.GBF_PREC_SPLIT_DF, "split_defect": abi.GBF_PREC_SPLIT_DEFECT}[form]
    steps = 12
    dom = Domain(m, None, st.K, st.phi, precision=p)
    assert gpu_lib.gbf_domain_uses_tma(dom.h) == 1
    dom.set_outputs(abi.GBF_OUT_MASS | abi.GBF_OUT_CFL, steps)
    dom.upload(st["P1"], st["S2"])
    refs = []
    for _ in range(steps):
        refs.append(cfl_reference(m, dom.download("P1"), dom.download("S2"), st.K, st.phi))
        dom.step(1)
    cfl = dom.cfl_history(steps)
    assert cfl.shape == (steps, 2) and dom.status() == abi.GBF_OK
    ref = np.array(refs)
    assert (ref > 1e-9).all()  # both phases mobile
    # FP32 state and mobilities: 2e-3 relative; CFL numbers below 1e-12 (a
    # trace of DNAPL, zero in FP32) count as zero
    np.testing.assert_allclose(cfl, ref, rtol=2e-3, atol=1e-12)
    # the mass history is unaffected by CFL recording
    dom2 = Domain(m, None, st.K, st.phi, precision=p)
    dom2.set_outputs(abi.GBF_OUT_MASS, steps)
    dom2.upload(st["P1"], st["S2"])
    dom2.step(steps)
    assert np.array_equal(dom2.mass_history(steps), dom.mass_history(steps))
    dom.close()
    dom2.close()


def test_ensemble_cfl_equals_single_domains(gpu_lib, abi, pkg):
    from test_gpu_ensemble import members, mods
    E, D = mods(pkg)
    mems = members(abi, gpu_lib)
    steps = 6
    for shape in (0, 3, 4, 5):
        ens = E.Ensemble(mems, precision=abi.GBF_PREC_SPLIT_DF)
        ens.set_tuning(shape, 0, 0)
        ens.set_outputs(abi.GBF_OUT_MASS | abi.GBF_OUT_CFL, steps)
        ens.upload_initial()
        ens.step(steps)
        cfl = ens.cfl_history(steps)
        assert cfl.shape == (steps, len(mems), 2)
        for r, mem in enumerate(mems):
            d = D.Domain(mem.model, None, mem.K, mem.phi, precision=abi.GBF_PREC_SPLIT_DF)
            d.set_outputs(abi.GBF_OUT_MASS | abi.GBF_OUT_CFL, steps)
            d.upload(*mem.initial_state())
            d.step(steps)
            assert np.array_equal(cfl[:, r, :], d.cfl_history(steps)), (shape, r)
            d.close()
        ens.close()
