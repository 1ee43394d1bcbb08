// gbf_f64_cell.cuh — per-cell device code of the plain FP64 step, shared by
// the single-domain kernels (gbf_f64.cu) and the batched ones (gbf_ensemble.cu).
#pragma once

#include <math.h>

#include "gbf_domain.h"

__device__ __forceinline__ int gbf_media_at(const gbf_cells& c, size_t idx) { return c.media ? c.media[idx] : 0; }

// Pass 1 at cell c (every cell): Brooks-Corey kr from one log and two exp
// (cpu.cpp:57-74), densities, L = Xi ro, ln S_e; optionally the reference's
// P2/Xi arrays and a2's velocities (cpu.cpp:77-160).
__device__ __forceinline__ void gbf_f64_props_cell(const gbf_model& m, const GbfDerived& d, const gbf_cells& cells,
                                                   const GbfF64Step& s, int flags, const GbfGeo& g, size_t c) {
  const int md = gbf_media_at(cells, c);
  const double K = cells.K ? (double)cells.K[c] : m.K[md];
  const double S2 = s.S[c], P1 = s.P[c];
  const double S_e = (1. - S2 - m.S_wr[md]) * d.inv_1mswr[md];
  const double l = log(S_e);
  const double k1 = exp(d.e1[md] * l);
  const double k2 = (1. - S_e) * (1. - S_e) * (1. - exp(d.e2[md] * l));
  const double Xi1 = K * k1 * d.neg_inv_mu1;
  const double Xi2 = K * k2 * d.neg_inv_mu2;
  const double ro1 = m.ro01 * (1. + m.beta1 * (P1 - m.P_atm));
  const double ro2 = m.ro02 * (1. + m.beta2 * (P1 - m.P_atm));  // P2 = P1 (P_k = 0, cpu.cpp:63)
  s.L1[c] = Xi1 * ro1;
  s.L2[c] = Xi2 * ro2;
  s.ro1[c] = ro1;
  s.ro2[c] = ro2;
  s.lnSe[c] = l;
  if (flags & GBF_PF_WRITE_XI_P2) {
    s.Xi1[c] = Xi1;
    s.Xi2[c] = Xi2;
    s.P2[c] = P1;
  }
  if (flags & GBF_PF_WRITE_U) {
    const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / g.pl);
    const double* P = s.P;
    const double dx = (i == 0) ? (P[c + 1] - P1) / m.h1
                    : (i == g.nx - 1) ? (P1 - P[c - 1]) / m.h1 : (P[c + 1] - P[c - 1]) / (2. * m.h1);
    const double dy = (j == 0) ? (P[c + g.nx] - P1) / m.h2
                    : (j == g.ny - 1) ? (P1 - P[c - g.nx]) / m.h2 : (P[c + g.nx] - P[c - g.nx]) / (2. * m.h2);
    const double dz = (k == 0) ? (P[c + g.pl] - P1) / m.h3
                    : (k == g.nz - 1) ? (P1 - P[c - g.pl]) / m.h3 : (P[c + g.pl] - P[c - g.pl]) / (2. * m.h3);
    s.u1x[c] = Xi1 * dx;
    s.u2x[c] = Xi2 * dx;
    s.u1y[c] = m.kv * Xi1 * (dy - ro1 * m.g);
    s.u2y[c] = m.kv * Xi2 * (dy - ro2 * m.g);
    s.u1z[c] = Xi1 * dz;
    s.u2z[c] = Xi2 * dz;
  }
}

// Donor-cell flux difference of one direction: the reference's
// ((x2+|x2|)/2 - (x1-|x1|)/2)(-1)L_c - (x1+|x1|)/2 (-1)L_m + (x2-|x2|)/2 (-1)L_p
// (cpu.cpp:260-262) with (x+|x|)/2 = max(x, 0) and (x-|x|)/2 = min(x, 0), which are exact.
__device__ __forceinline__ double gbf_donor(double x1, double x2, double Lc, double Lm, double Lp) {
  const double x2p = x2 > 0. ? x2 : 0., x2m = x2 > 0. ? 0. : x2;
  const double x1p = x1 > 0. ? x1 : 0., x1m = x1 > 0. ? 0. : x1;
  return (x1p * Lm - (x2p - x1m) * Lc) - x2m * Lp;
}

// Newton for (P1, S2) from the phase masses (cpu.cpp:293-320); the first
// iteration reuses ln(S_e) of pass 1; stops at round-off (model.newton_tol)
// or after model.newton_iterations.
//
// After a step dx = (dP, dS) the residual is the Taylor remainder of F, which
// for this system is R1 = -rho01 beta1 dP dS (F1 is bilinear in P, S) and
// R2 = rho02 beta2 (dP dS + g'' dS^2 / 2) with g(S) = P_k(S) S; the next step
// would be J^-1 R. When that predicted step is below tol / 1000 relative to
// S and to P the iteration stops without computing it (relative in S too:
// near a rate source S can be 1e-10 and its mass must keep round-off
// accuracy); the usual case
// at stable time steps, where one step already lands within round-off (with
// equal compressibilities the dP dS terms cancel in the P component). g'' is
// taken at the start point with a factor 2 for its change over the step.
__device__ __forceinline__ void gbf_f64_newton(const gbf_model& m, const GbfDerived& d, int md, double lnSe0,
                                               double roS1, double roS2, double& P1, double& S2) {
  const double tol = m.newton_tol, swr = m.S_wr[md], pd = m.P_d[md];
  for (int w = 1; w <= m.newton_iterations; w++) {
    const double S_e = (1. - S2 - swr) * d.inv_1mswr[md];
    const double l = (w == 1) ? lnSe0 : log(S_e);
    const double P_k = pd * exp(d.m_inv_lam[md] * l);
    const double PkS = P_k * d.inv_lam_1mswr[md] / S_e;  // S_e^(-1/lambda - 1) P_d / (lambda (1 - S_wr))
    const double t1 = 1. + m.beta1 * (P1 - m.P_atm);
    const double t2 = 1. + m.beta2 * (P1 + P_k - m.P_atm);
    const double F1 = m.ro01 * t1 * (1. - S2) - roS1;
    const double F2 = m.ro02 * t2 * S2 - roS2;
    const double F1P = m.ro01 * m.beta1 * (1. - S2);
    const double F2P = m.ro02 * m.beta2 * S2;
    const double F1S = -m.ro01 * t1;
    const double F2S = m.ro02 * (t2 + m.beta2 * S2 * PkS);
    const double inv_det = 1. / (F1P * F2S - F1S * F2P);
    const double dP = inv_det * (F2S * F1 - F1S * F2);
    const double dS = inv_det * (F1P * F2 - F2P * F1);
    const double S0 = S2;
    P1 -= dP;
    S2 -= dS;
    if (tol > 0. && fabs(dS) <= tol && fabs(dP) <= tol * fabs(P1)) break;
    if (tol > 0.) {  // the predicted next step, from the remainder
      const double Pk2 = PkS * (1. - d.m_inv_lam[md]) * d.inv_1mswr[md] / S_e;  // P_k'' = P_k' (1 / lambda + 1) / ((1 - S_wr) S_e)
      const double g2 = 0.5 * dS * dS * 2. * fabs(Pk2 * S0 + 2. * PkS) * m.ro02 * m.beta2;  // |g'' part of R2|
      const double R1 = -m.ro01 * m.beta1 * dP * dS, R2 = m.ro02 * m.beta2 * dP * dS;   // the dP dS parts, signed
      const double eP = fabs(inv_det * (F2S * R1 - F1S * R2)) + fabs(inv_det * F1S) * g2;
      const double eS = fabs(inv_det * (F1P * R2 - F2P * R1)) + fabs(inv_det * F1P) * g2;
      if (eS <= 1e-3 * tol * fabs(S2) && eP <= 1e-3 * tol * fabs(P1)) break;  // relative: S may be tiny
    }
  }
}

// Pass 2 at interior cell (i, j, k): face fluxes with gravity and the mass
// update (cpu.cpp:218-291), then the Newton step; writes the next state.
// Adds phi * A to the mass sums and flags non-finite results.
__device__ __forceinline__ void gbf_f64_flux_newton_cell(const gbf_model& m, const GbfDerived& d,
                                                         const gbf_cells& cells, const GbfF64Step& s,
                                                         const GbfGeo& g, int i, int j, int k, double& msum1,
                                                         double& msum2, unsigned& bad) {
  const size_t c = gbf_idx(g, i, j, k), nx = g.nx, pl = g.pl;
  const bool noflow_bottom = (m.bc_mode == GBF_BC_HYDROSTATIC_SIDES) && (j == g.ny - 2);
  const int md = gbf_media_at(cells, c);
  const double phi = cells.phi ? (double)cells.phi[c] : m.m[md];
  const double* P = s.P;
  const double Pc = P[c];
  // face potentials (P2 = P1 in the flux step)
  const double x1 = (P[c - 1] - Pc) * d.inv_h1, x2 = (Pc - P[c + 1]) * d.inv_h1;
  const double yb1 = (P[c - nx] - Pc) * d.inv_h2, yb2 = (Pc - P[c + nx]) * d.inv_h2;
  const double z1 = (P[c - pl] - Pc) * d.inv_h3, z2 = (Pc - P[c + pl]) * d.inv_h3;
  const double ro1 = s.ro1[c], ro2 = s.ro2[c];
  const double rg1 = ro1 * m.g, rg2 = ro2 * m.g;
  const double y1_1 = yb1 + rg1, y1_2 = yb1 + rg2;
  const double y2_1 = noflow_bottom ? 0. : yb2 + rg1;
  const double y2_2 = noflow_bottom ? 0. : yb2 + rg2;
  const double* L1 = s.L1;
  const double* L2 = s.L2;
  const double L1c = L1[c], L2c = L2[c];
  const double f = gbf_donor(x1, x2, L1c, L1[c - 1], L1[c + 1]) * d.inv_h1 +
                   m.kv * gbf_donor(y1_1, y2_1, L1c, L1[c - nx], L1[c + nx]) * d.inv_h2 +
                   gbf_donor(z1, z2, L1c, L1[c - pl], L1[c + pl]) * d.inv_h3;
  const double gsum = gbf_donor(x1, x2, L2c, L2[c - 1], L2[c + 1]) * d.inv_h1 +
                      m.kv * gbf_donor(y1_2, y2_2, L2c, L2[c - nx], L2[c + nx]) * d.inv_h2 +
                      gbf_donor(z1, z2, L2c, L2[c - pl], L2[c + pl]) * d.inv_h3;
  const double S2 = s.S[c];
  const double roS1 = ro1 * (1. - S2), roS2 = ro2 * S2;
  const double dtphi = m.dt / phi;
  const double A1 = roS1 - dtphi * f;
  double A2 = roS2 - dtphi * gsum;
  if (d.src != 0. && j == 1 && gbf_in_rate_patch(m, i, k)) A2 += dtphi * d.src;
  if (s.roS1) {
    s.roS1[c] = A1;
    s.roS2[c] = A2;
    s.roS1_old[c] = roS1;
    s.roS2_old[c] = roS2;
  }
  msum1 += phi * A1;
  msum2 += phi * A2;
  double Pn = Pc, Sn = S2;
  gbf_f64_newton(m, d, md, s.lnSe[c], A1, A2, Pn, Sn);
  if (!isfinite(Pn) || !isfinite(Sn)) bad = 1;
  s.Pn[c] = Pn;
  s.Sn[c] = Sn;
}

// Face pass at boundary cell number t (gbf_boundary_cell order).
__device__ __forceinline__ void gbf_f64_boundary_cell(const gbf_model& m, const GbfF64Step& s, const GbfGeo& g,
                                                      size_t t) {
  int i, j, k;
  gbf_boundary_cell(g, t, i, j, k);
  const size_t c = gbf_idx(g, i, j, k);
  const double* ro1 = s.ro1;
  auto ro1_top = [ro1, &g](int ii) { return ro1[(size_t)ii + (size_t)g.nx]; };
  s.Sn[c] = gbf_sweep_S<double>(m, g, s.Sn, s.S, i, j, k);
  s.Pn[c] = gbf_sweep_P<double>(m, g, s.Pn, s.P, i, j, k, ro1_top);
}

// Sum of warp values of the block into out[0..1] (thread 0), fixed order.
template <int NT>
__device__ __forceinline__ void gbf_block_sum2(double a, double b, double V, double* out) {
  __shared__ double red[2][NT / 32];
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_down_sync(0xffffffffu, a, o);
    b += __shfl_down_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { red[0][w] = a; red[1][w] = b; }
  __syncthreads();
  if (threadIdx.x == 0) {
    double x = 0., y = 0.;
    for (int q = 0; q < NT / 32; q++) { x += red[0][q]; y += red[1][q]; }
    out[0] = x * V;
    out[1] = y * V;
  }
  __syncthreads();
}
