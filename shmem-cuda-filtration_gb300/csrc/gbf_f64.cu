// gbf_f64.cu — plain FP64 step, fused into two passes plus a face pass.
//
// GB300 executes FP64 at about 1/64 of its FP32 rate (measured 1.2 TFLOP/s
// DFMA against 6.4 TB/s of HBM), so a plain FP64 step is bound by the FP64
// pipe, not by memory: the design minimises FP64 instructions per cell and
// spends bytes freely to do so.
//   pass 1 (k_f64_props, every cell): one log and two exp per cell for the
//     Brooks-Corey relative permeabilities (cpu.cpp:57-74), the densities,
//     and L = Xi * ro per phase; ln(S_e) is kept for the Newton step.
//   pass 2 (k_f64_flux_newton, interior cells): upwinded face fluxes with
//     gravity (cpu.cpp:218-291) and the 2x2 Newton (cpu.cpp:293-320) fused;
//     the first iteration reuses ln(S_e) from pass 1 and the iteration stops
//     once the update is at round-off (model.newton_tol), at most
//     model.newton_iterations times. Writes the next state (ping-pong) and,
//     optionally, per-block phase-mass partial sums.
//   face pass (k_f64_boundary): the reference's sweep-ordered boundary
//     values (cpu.cpp:44-54, 323-403) into the next state.
// Every cell's properties are computed once per step (no halo recomputation),
// which is what an FP64-bound kernel wants.
#include <math.h>

#include "gbf_domain.h"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int media_at(const gbf_cells& c, size_t idx) { return c.media ? c.media[idx] : 0; }

__global__ void __launch_bounds__(kThreads) k_f64_props(const gbf_model m, const GbfDerived d, const gbf_cells cells,
                                                        const GbfF64Step s, const int flags) {
  const GbfGeo g = gbf_geo(m);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.n; c += (size_t)gridDim.x * blockDim.x) {
    const int md = media_at(cells, c);
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
    if (flags & GBF_PF_WRITE_U) {  // a2 (cpu.cpp:77-160) from this cell's Xi, ro and the P stencil
      const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / g.pl);
      const double* P = s.P;
      double dx = (i == 0) ? (P[c + 1] - P1) / m.h1
                : (i == g.nx - 1) ? (P1 - P[c - 1]) / m.h1 : (P[c + 1] - P[c - 1]) / (2. * m.h1);
      double dy = (j == 0) ? (P[c + g.nx] - P1) / m.h2
                : (j == g.ny - 1) ? (P1 - P[c - g.nx]) / m.h2 : (P[c + g.nx] - P[c - g.nx]) / (2. * m.h2);
      double dz = (k == 0) ? (P[c + g.pl] - P1) / m.h3
                : (k == g.nz - 1) ? (P1 - P[c - g.pl]) / m.h3 : (P[c + g.pl] - P[c - g.pl]) / (2. * m.h3);
      s.u1x[c] = Xi1 * dx;
      s.u2x[c] = Xi2 * dx;
      s.u1y[c] = m.kv * Xi1 * (dy - ro1 * m.g);
      s.u2y[c] = m.kv * Xi2 * (dy - ro2 * m.g);
      s.u1z[c] = Xi1 * dz;
      s.u2z[c] = Xi2 * dz;
    }
  }
}

// Donor-cell flux difference of one direction: the reference's
// ((x2+|x2|)/2 - (x1-|x1|)/2)(-1)L_c - (x1+|x1|)/2 (-1)L_m + (x2-|x2|)/2 (-1)L_p
// with (x+|x|)/2 = max(x, 0) and (x-|x|)/2 = min(x, 0), which are exact.
__device__ __forceinline__ double donor(double x1, double x2, double Lc, double Lm, double Lp) {
  const double x2p = x2 > 0. ? x2 : 0., x2m = x2 > 0. ? 0. : x2;
  const double x1p = x1 > 0. ? x1 : 0., x1m = x1 > 0. ? 0. : x1;
  return (x1p * Lm - (x2p - x1m) * Lc) - x2m * Lp;
}

struct NewtonConsts {
  double swr, pd, lam, m_inv_lam, inv_1mswr, inv_lam_1mswr;
};

// Newton for (P1, S2) given the phase masses (cpu.cpp:293-320); the first
// iteration uses ln(S_e) of the current state from pass 1.
__device__ __forceinline__ void newton(const gbf_model& m, const NewtonConsts& q, double lnSe0, double roS1,
                                       double roS2, double& P1, double& S2) {
  const double tol = m.newton_tol;
  for (int w = 1; w <= m.newton_iterations; w++) {
    const double S_e = (1. - S2 - q.swr) * q.inv_1mswr;
    const double l = (w == 1) ? lnSe0 : log(S_e);
    const double P_k = q.pd * exp(q.m_inv_lam * l);
    const double PkS = P_k * q.inv_lam_1mswr / S_e;  // = S_e^(-1/lambda - 1) P_d / (lambda (1 - S_wr))
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
    P1 -= dP;
    S2 -= dS;
    if (tol > 0. && fabs(dS) <= tol && fabs(dP) <= tol * fabs(P1)) break;
  }
}

__global__ void __launch_bounds__(kThreads) k_f64_flux_newton(const gbf_model m, const GbfDerived d,
                                                              const gbf_cells cells, const GbfF64Step s) {
  const GbfGeo g = gbf_geo(m);
  const size_t ix = (size_t)g.nx - 2, iy = (size_t)g.ny - 2;
  const size_t nint = ix * iy * (size_t)(g.nz - 2);
  const bool noflow_bottom = (m.bc_mode == GBF_BC_HYDROSTATIC_SIDES);
  double msum1 = 0., msum2 = 0.;
  unsigned bad = 0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nint; t += (size_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % ix), j = 1 + (int)((t / ix) % iy), k = 1 + (int)(t / (ix * iy));
    const size_t c = gbf_idx(g, i, j, k), nx = g.nx, pl = g.pl;
    const int md = media_at(cells, c);
    const double phi = cells.phi ? (double)cells.phi[c] : m.m[md];
    const double* P = s.P;
    const double Pc = P[c];
    // face potentials (P2 = P1 in the flux step)
    const double x1 = (P[c - 1] - Pc) * d.inv_h1, x2 = (Pc - P[c + 1]) * d.inv_h1;
    const double yb1 = (P[c - nx] - Pc) * d.inv_h2, yb2 = (noflow_bottom && j == g.ny - 2) ? 0. : (Pc - P[c + nx]) * d.inv_h2;
    const double z1 = (P[c - pl] - Pc) * d.inv_h3, z2 = (Pc - P[c + pl]) * d.inv_h3;
    const double ro1 = s.ro1[c], ro2 = s.ro2[c];
    const double rg1 = ro1 * m.g, rg2 = ro2 * m.g;
    const double y1_1 = yb1 + rg1, y1_2 = yb1 + rg2;
    const double y2_1 = (noflow_bottom && j == g.ny - 2) ? 0. : yb2 + rg1;
    const double y2_2 = (noflow_bottom && j == g.ny - 2) ? 0. : yb2 + rg2;
    const double* L1 = s.L1;
    const double* L2 = s.L2;
    const double L1c = L1[c], L2c = L2[c];
    const double f = donor(x1, x2, L1c, L1[c - 1], L1[c + 1]) * d.inv_h1 +
                     m.kv * donor(y1_1, y2_1, L1c, L1[c - nx], L1[c + nx]) * d.inv_h2 +
                     donor(z1, z2, L1c, L1[c - pl], L1[c + pl]) * d.inv_h3;
    const double gsum = donor(x1, x2, L2c, L2[c - 1], L2[c + 1]) * d.inv_h1 +
                        m.kv * donor(y1_2, y2_2, L2c, L2[c - nx], L2[c + nx]) * d.inv_h2 +
                        donor(z1, z2, L2c, L2[c - pl], L2[c + pl]) * d.inv_h3;
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
    if (s.mass_partials) {
      msum1 += phi * A1;
      msum2 += phi * A2;
    }
    NewtonConsts q;
    q.swr = m.S_wr[md]; q.pd = m.P_d[md]; q.lam = m.lambda[md]; q.m_inv_lam = d.m_inv_lam[md];
    q.inv_1mswr = d.inv_1mswr[md]; q.inv_lam_1mswr = d.inv_lam_1mswr[md];
    double Pn = Pc, Sn = S2;
    newton(m, q, s.lnSe[c], A1, A2, Pn, Sn);
    if (!isfinite(Pn) || !isfinite(Sn)) bad = 1;
    s.Pn[c] = Pn;
    s.Sn[c] = Sn;
  }
  if (bad) atomicOr(s.status, GBF_DEV_NONFINITE);
  if (s.mass_partials) {  // deterministic per-block partials (fixed reduction order)
    __shared__ double red[2][kThreads / 32];
    for (int o = 16; o > 0; o >>= 1) {
      msum1 += __shfl_down_sync(0xffffffffu, msum1, o);
      msum2 += __shfl_down_sync(0xffffffffu, msum2, o);
    }
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) { red[0][w] = msum1; red[1][w] = msum2; }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0., b = 0.;
      for (int q = 0; q < kThreads / 32; q++) { a += red[0][q]; b += red[1][q]; }
      s.mass_partials[2 * blockIdx.x] = a * d.V;
      s.mass_partials[2 * blockIdx.x + 1] = b * d.V;
    }
  }
}

__global__ void __launch_bounds__(kThreads) k_f64_boundary(const gbf_model m, const GbfF64Step s) {
  const GbfGeo g = gbf_geo(m);
  const size_t nb = gbf_boundary_count(g);
  const double* ro1 = s.ro1;
  auto ro1_top = [ro1, &g](int i) { return ro1[(size_t)i + (size_t)g.nx]; };
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nb; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    gbf_boundary_cell(g, t, i, j, k);
    const size_t c = gbf_idx(g, i, j, k);
    s.Sn[c] = gbf_sweep_S<double>(m, g, s.Sn, s.S, i, j, k);
    s.Pn[c] = gbf_sweep_P<double>(m, g, s.Pn, s.P, i, j, k, ro1_top);
  }
}

// Sum the per-block partials in a fixed order (one block).
__global__ void k_mass_tail(const double* partials, int nblocks, double* out) {
  __shared__ double red[2][256];
  double a = 0., b = 0.;
  for (int q = threadIdx.x; q < nblocks; q += blockDim.x) { a += partials[2 * q]; b += partials[2 * q + 1]; }
  red[0][threadIdx.x] = a;
  red[1][threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) { red[0][threadIdx.x] += red[0][threadIdx.x + o]; red[1][threadIdx.x] += red[1][threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[0] = red[0][0]; out[1] = red[1][0]; }
}

}  // namespace

unsigned gbf_f64_flux_grid(const gbf_model& m) {
  size_t nint = (size_t)(m.nx - 2) * (m.ny - 2) * (m.nz - 2);
  return gbf_grid_for(nint, kThreads, 4);
}

int gbf_f64_launch_step(const gbf_model& m, const GbfDerived& d, const gbf_cells& cells, const GbfF64Step& s,
                        int props_flags, double* mass_out, cudaStream_t st, GbfTimer* tm) {
  const GbfGeo g = gbf_geo(m);
  cudaEvent_t e = gbf_timer_begin(tm, st);
  k_f64_props<<<gbf_grid_for(g.n, kThreads, 4), kThreads, 0, st>>>(m, d, cells, s, props_flags);
  gbf_timer_end(tm, GBF_K_PROPS, e, st);
  const unsigned fg = gbf_f64_flux_grid(m);
  e = gbf_timer_begin(tm, st);
  k_f64_flux_newton<<<fg, kThreads, 0, st>>>(m, d, cells, s);
  gbf_timer_end(tm, GBF_K_FLUX_NEWTON, e, st);
  e = gbf_timer_begin(tm, st);
  k_f64_boundary<<<gbf_grid_for(gbf_boundary_count(g), kThreads, 4), kThreads, 0, st>>>(m, s);
  gbf_timer_end(tm, GBF_K_BOUNDARY, e, st);
  if (s.mass_partials && mass_out) {
    e = gbf_timer_begin(tm, st);
    k_mass_tail<<<1, 256, 0, st>>>(s.mass_partials, (int)fg, mass_out);
    gbf_timer_end(tm, GBF_K_MASS_TAIL, e, st);
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? GBF_OK : gbf_cuda_check(err, "gbf_f64_launch_step");
}
