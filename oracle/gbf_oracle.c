/*
 * gbf_oracle.c — CPU oracle for the two-phase flow hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker: only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg may load it.
 * The product path (libgbflow) never links or calls it.
 *
 * It is a serial FP64 restatement of the reference CPU backend, written with
 * the same operation order so that, compiled with -O2 -ffp-contract=off, it
 * reproduces the reference bit for bit in reference mode (pinned by
 * tests/test_oracle.py against the reference's cpu.cpp compiled from its own
 * sources, and against committed golden fixtures generated from it):
 *
 *   orc_props       cpu.cpp:3-15, 57-74    (ro_P2_Xi_calculation)
 *   orc_velocity    cpu.cpp:17-24, 77-160  (u_calculation)
 *   orc_mass        cpu.cpp:26-33, 218-291 (roS_calculation -> assign_rS_nr)
 *   orc_newton      cpu.cpp:35-42, 293-320 (P1_S2_calculation -> Newton)
 *   orc_boundary    cpu.cpp:44-54, 323-403 (boundary_conditions)
 *   orc_step        main.cpp:83-94         (time_step_function, single domain)
 *   orc_initial     main.cpp:97-138        (initial_data, single domain)
 *
 * The loops of orc_props/velocity/mass/newton run in parallel over i with
 * OpenMP (each iteration writes only its own cells and reads arrays the loop
 * does not write, so the result does not depend on the thread count); the
 * boundary sweep and the mass sums stay serial.
 *
 * Extensions (all off in reference mode, see gbf_model): per-cell K and
 * porosity, vertical anisotropy kv, mass-rate injection, hydrostatic side
 * boundaries with a no-flow bottom, and a Newton tolerance stop.
 */
#include <math.h>
#include <stddef.h>
#include <string.h>

#include "../include/gbflow.h"

#define ORC_IDX(i, j, k) ((size_t)(i) + (size_t)(j) * (size_t)nx + (size_t)(k) * (size_t)nx * (size_t)ny)

static int media_of(const gbf_cells* c, size_t idx) { return (c && c->media) ? c->media[idx] : 0; }
static double K_of(const gbf_model* m, const gbf_cells* c, size_t idx, int media) {
  return (c && c->K) ? (double)c->K[idx] : m->K[media];
}
static double phi_of(const gbf_model* m, const gbf_cells* c, size_t idx, int media) {
  return (c && c->phi) ? (double)c->phi[idx] : m->m[media];
}

/* Interior test of cpu.cpp:220 / :295 (single domain: localNx = NX). */
static int is_interior(const gbf_model* m, int i, int j, int k) {
  return (i != 0) && (i != m->nx - 1) && (j != 0) && (j != m->ny - 1) &&
         (((k != 0) && (k != m->nz - 1)) || (m->nz < 2));
}

/* Top-centre patch membership: reference form |I - NX/2| <= source (cpu.cpp:346). */
static int in_dirichlet_patch(const gbf_model* m, int i, int k) {
  return (i >= m->nx / 2 - m->source) && (i <= m->nx / 2 + m->source) &&
         (k >= m->nz / 2 - m->source) && (k <= m->nz / 2 + m->source);
}
/* Rate-injection patch: n x n cells centred like the reference patch
   (n = 2s+1 gives exactly the reference's cells). */
int orc_in_rate_patch(const gbf_model* m, int i, int k) {
  int n = m->rate_cells;
  int i0 = m->nx / 2 - n / 2, k0 = m->nz / 2 - n / 2;
  return (i >= i0) && (i < i0 + n) && (k >= k0) && (k < k0 + n);
}

/* a1: Brooks-Corey relative permeabilities, P2 = P1 (P_k = 0), mobilities Xi,
   densities; every cell (cpu.cpp:57-74). */
void orc_props(const gbf_model* m, const gbf_cells* cells, gbf_arrays a) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz; k++) {
        size_t c = ORC_IDX(i, j, k);
        int md = media_of(cells, c);
        double K = K_of(m, cells, c, md);
        double S_e = (1. - a.S2[c] - m->S_wr[md]) / (1. - m->S_wr[md]);
        double k1 = pow(S_e, (2. + 3. * m->lambda[md]) / m->lambda[md]);
        double k2 = (1. - S_e) * (1. - S_e) * (1 - pow(S_e, (2. + m->lambda[md]) / m->lambda[md]));
        double P_k = 0;
        a.P2[c] = a.P1[c] + P_k;
        a.Xi1[c] = -1. * K * k1 / m->mu1;
        a.Xi2[c] = -1. * K * k2 / m->mu2;
        a.ro1[c] = m->ro01 * (1. + (m->beta1) * (a.P1[c] - m->P_atm));
        a.ro2[c] = m->ro02 * (1. + (m->beta2) * (a.P2[c] - m->P_atm));
      }
}

/* a2: cell-centred phase velocities, one-sided on the faces (cpu.cpp:77-160).
   The vertical component carries the anisotropy factor kv. */
void orc_velocity(const gbf_model* m, gbf_arrays a) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const double kv = m->kv;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz; k++) {
        size_t c = ORC_IDX(i, j, k);
        if (nx > 2) {
          if (i == 0) {
            a.u1x[c] = a.Xi1[c] * (a.P1[c + 1] - a.P1[c]) / (m->h1);
            a.u2x[c] = a.Xi2[c] * (a.P2[c + 1] - a.P2[c]) / (m->h1);
          } else if (i == nx - 1) {
            a.u1x[c] = a.Xi1[c] * (a.P1[c] - a.P1[c - 1]) / (m->h1);
            a.u2x[c] = a.Xi2[c] * (a.P2[c] - a.P2[c - 1]) / (m->h1);
          } else {
            a.u1x[c] = a.Xi1[c] * ((a.P1[c + 1] - a.P1[c - 1]) / (2. * (m->h1)));
            a.u2x[c] = a.Xi2[c] * ((a.P2[c + 1] - a.P2[c - 1]) / (2. * (m->h1)));
          }
        } else {
          a.u1x[c] = 0;
          a.u2x[c] = 0;
        }
        if (ny > 2) {
          size_t up = c - (size_t)nx, dn = c + (size_t)nx;
          if (j == 0) {
            a.u1y[c] = kv * a.Xi1[c] * ((a.P1[dn] - a.P1[c]) / (m->h2) - a.ro1[c] * m->g);
            a.u2y[c] = kv * a.Xi2[c] * ((a.P2[dn] - a.P2[c]) / (m->h2) - a.ro2[c] * m->g);
          } else if (j == ny - 1) {
            a.u1y[c] = kv * a.Xi1[c] * ((a.P1[c] - a.P1[up]) / (m->h2) - a.ro1[c] * m->g);
            a.u2y[c] = kv * a.Xi2[c] * ((a.P2[c] - a.P2[up]) / (m->h2) - a.ro2[c] * m->g);
          } else {
            a.u1y[c] = kv * a.Xi1[c] * ((a.P1[dn] - a.P1[up]) / (2. * (m->h2)) - a.ro1[c] * m->g);
            a.u2y[c] = kv * a.Xi2[c] * ((a.P2[dn] - a.P2[up]) / (2. * (m->h2)) - a.ro2[c] * m->g);
          }
        } else {
          a.u1y[c] = 0;
          a.u2y[c] = 0;
        }
        if (nz > 2) {
          size_t pl = (size_t)nx * (size_t)ny;
          if (k == 0) {
            a.u1z[c] = a.Xi1[c] * (a.P1[c + pl] - a.P1[c]) / (m->h3);
            a.u2z[c] = a.Xi2[c] * (a.P2[c + pl] - a.P2[c]) / (m->h3);
          } else if (k == nz - 1) {
            a.u1z[c] = a.Xi1[c] * (a.P1[c] - a.P1[c - pl]) / (m->h3);
            a.u2z[c] = a.Xi2[c] * (a.P2[c] - a.P2[c - pl]) / (m->h3);
          } else {
            a.u1z[c] = a.Xi1[c] * ((a.P1[c + pl] - a.P1[c - pl]) / (2. * (m->h3)));
            a.u2z[c] = a.Xi2[c] * ((a.P2[c + pl] - a.P2[c - pl]) / (2. * (m->h3)));
          }
        } else {
          a.u1z[c] = 0;
          a.u2z[c] = 0;
        }
      }
}

/* Upwinded (donor-cell) divergence of one direction, the reference's expression
   (cpu.cpp:260-262): x2/x1 are the potentials on the +/- faces; (Xc, rc),
   (Xm, rm), (Xp, rp) the mobility Xi and density ro at the centre, minus and
   plus neighbours, multiplied in the reference's left-to-right order. */
static double upwind_div(double x1, double x2, double Xc, double rc, double Xm, double rm,
                         double Xp, double rp, double h);

/* Experiment switch (off by default; the tests only): what the split forms'
   FP32 flux stage does to the phase masses in an otherwise FP64 scheme.
   1: every upwinded mobility Xi*ro rounded to FP32 before it multiplies the
      face potential, and nothing else.
   2: the same except on the DNAPL face between a Dirichlet patch cell and the
      j = 1 cell below it, which keeps its FP64 mobility (the split forms' FP64
      patch inflow).
   3: mobilities FP64 and the flux arithmetic FP32 as in the split forms: each
      face's upwinded flux (potential times mobility) rounded to FP32, each
      direction's in - out and its dt / h^2 weighting rounded, the cell's sum
      of the three rounded, the increment over phi rounded and added to the
      FP64 mass; the DNAPL flux through the Dirichlet patch faces stays FP64
      and is added apart, like the rate source.
   4: 3 with the split tile's remaining FP32 steps: mobilities rounded to FP32
      (but the patch faces' DNAPL one), and in y the minus face's product
      entering the difference unrounded (the tile's FMA) while the plus face's
      is rounded, so that a y face's flux differs by one rounding between its
      two cells. */
static int g_fp32_mobilities = 0;
void orc_set_fp32_mobilities(int on) { g_fp32_mobilities = on; }

/* The y-direction DNAPL divergence of a j = 1 cell under the Dirichlet patch
   at experiment level 2: FP32 mobilities on its plus face, FP64 on its minus
   (patch) face. */
static double upwind_div_patch(double x1, double x2, double Xc, double rc, double Xm, double rm,
                               double Xp, double rp, double h) {
  const double Lc = (float)(Xc * rc), Lp = (float)(Xp * rp);
  return ((x2 + fabs(x2)) / 2.0 * (-1) * Lc - (x1 - fabs(x1)) / 2.0 * (-1) * (Xc * rc) -
          (x1 + fabs(x1)) / 2.0 * (-1) * (Xm * rm) + (x2 - fabs(x2)) / 2.0 * (-1) * Lp) / h;
}

/* Experiment levels 3 and 4: the upwinded fluxes through the minus (F1) and
   plus (F2) faces as the split tile signs them, -(potential times mobility):
   h upwind_div = F2 - F1. */
static double mob(double X, double r, int r32) { return r32 ? (double)(float)(X * r) : X * r; }
static void face_fluxes(double x1, double x2, double Xc, double rc, double Xm, double rm, double Xp, double rp,
                        double* F1, double* F2) {
  const int r32 = g_fp32_mobilities == 4;
  *F1 = x1 >= 0 ? x1 * (-mob(Xm, rm, r32)) : x1 * (-mob(Xc, rc, r32));
  *F2 = x2 >= 0 ? x2 * (-mob(Xc, rc, r32)) : x2 * (-mob(Xp, rp, r32));
}
/* dt/h^2 (kv in y) times in - out, FP32 as the split tile forms it (fma_minus:
   the minus face's product unrounded inside the difference, level 4 in y). */
static float fp32_dir(double F1, double F2, double w, int fma_minus) {
  const float d = fma_minus ? (float)(F1 - (double)(float)F2) : (float)F1 - (float)F2;
  return d * (float)w;
}

static double upwind_div(double x1, double x2, double Xc, double rc, double Xm, double rm,
                         double Xp, double rp, double h) {
  if (g_fp32_mobilities == 1 || g_fp32_mobilities == 2) {
    const double Lc = (float)(Xc * rc), Lm = (float)(Xm * rm), Lp = (float)(Xp * rp);
    return (((x2 + fabs(x2)) / 2.0 - (x1 - fabs(x1)) / 2.0) * (-1) * Lc - (x1 + fabs(x1)) / 2.0 * (-1) * Lm +
            (x2 - fabs(x2)) / 2.0 * (-1) * Lp) / h;
  }
  return (((x2 + fabs(x2)) / 2.0 - (x1 - fabs(x1)) / 2.0) * (-1) * Xc * rc -
          (x1 + fabs(x1)) / 2.0 * (-1) * Xm * rm +
          (x2 - fabs(x2)) / 2.0 * (-1) * Xp * rp) / h;
}

/* a3: explicit phase-mass update on interior cells (cpu.cpp:218-291). */
void orc_mass(const gbf_model* m, const gbf_cells* cells, gbf_arrays a) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const size_t pl = (size_t)nx * (size_t)ny;
  const int noflow_bottom = (m->bc_mode == GBF_BC_HYDROSTATIC_SIDES);
  const double src = (m->source_mode == GBF_SOURCE_RATE && m->rate_cells > 0)
                         ? m->rate / (double)(m->rate_cells * m->rate_cells) / (m->h1 * m->h2 * m->h3)
                         : 0.0;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz; k++) {
        if (!is_interior(m, i, j, k)) continue;
        size_t c = ORC_IDX(i, j, k);
        int md = media_of(cells, c);
        double phi = phi_of(m, cells, c, md);
        double roS1 = a.ro1[c] * (1 - a.S2[c]);
        double roS2 = a.ro2[c] * a.S2[c];
        double P1 = a.P1[c], P2 = a.P2[c];
        double x1, x2, y1, y2, z1, z2, f1, f2, f3, g1, g2, g3;
        if (nz < 2) {
          f3 = 0;
          g3 = 0;
        } else {
          z2 = -(a.P1[c + pl] - P1) / m->h3;
          z1 = -(P1 - a.P1[c - pl]) / m->h3;
          f3 = upwind_div(z1, z2, a.Xi1[c], a.ro1[c], a.Xi1[c - pl], a.ro1[c - pl], a.Xi1[c + pl], a.ro1[c + pl], m->h3);
          z2 = -(a.P2[c + pl] - P2) / m->h3;
          z1 = -(P2 - a.P2[c - pl]) / m->h3;
          g3 = upwind_div(z1, z2, a.Xi2[c], a.ro2[c], a.Xi2[c - pl], a.ro2[c - pl], a.Xi2[c + pl], a.ro2[c + pl], m->h3);
        }
        x2 = -(a.P1[c + 1] - P1) / m->h1;
        x1 = -(P1 - a.P1[c - 1]) / m->h1;
        y2 = -(a.P1[c + nx] - P1) / m->h2 + a.ro1[c] * m->g;
        y1 = -(P1 - a.P1[c - nx]) / m->h2 + a.ro1[c] * m->g;
        if (noflow_bottom && j == ny - 2) y2 = 0;
        f1 = upwind_div(x1, x2, a.Xi1[c], a.ro1[c], a.Xi1[c - 1], a.ro1[c - 1], a.Xi1[c + 1], a.ro1[c + 1], m->h1);
        f2 = m->kv * upwind_div(y1, y2, a.Xi1[c], a.ro1[c], a.Xi1[c - nx], a.ro1[c - nx], a.Xi1[c + nx], a.ro1[c + nx], m->h2);
        x2 = -(a.P2[c + 1] - P2) / m->h1;
        x1 = -(P2 - a.P2[c - 1]) / m->h1;
        y2 = -(a.P2[c + nx] - P2) / m->h2 + a.ro2[c] * m->g;
        y1 = -(P2 - a.P2[c - nx]) / m->h2 + a.ro2[c] * m->g;
        if (noflow_bottom && j == ny - 2) y2 = 0;
        g1 = upwind_div(x1, x2, a.Xi2[c], a.ro2[c], a.Xi2[c - 1], a.ro2[c - 1], a.Xi2[c + 1], a.ro2[c + 1], m->h1);
        if (g_fp32_mobilities == 2 && j == 1 && m->source_mode == GBF_SOURCE_DIRICHLET_PATCH && in_dirichlet_patch(m, i, k))
          g2 = m->kv * upwind_div_patch(y1, y2, a.Xi2[c], a.ro2[c], a.Xi2[c - nx], a.ro2[c - nx], a.Xi2[c + nx],
                                        a.ro2[c + nx], m->h2);
        else
          g2 = m->kv * upwind_div(y1, y2, a.Xi2[c], a.ro2[c], a.Xi2[c - nx], a.ro2[c - nx], a.Xi2[c + nx], a.ro2[c + nx], m->h2);
        if (g_fp32_mobilities == 3 || g_fp32_mobilities == 4) {  /* FP32 flux arithmetic, FP64 patch inflow */
          const int fy = g_fp32_mobilities == 4;
          const int ptop = j == 1 && m->source_mode == GBF_SOURCE_DIRICHLET_PATCH && in_dirichlet_patch(m, i, k);
          double F1, F2;
          float s1 = 0.f, s2 = 0.f;
          double pin = 0.0;
          if (nz >= 2) {
            z2 = -(a.P1[c + pl] - P1) / m->h3;
            z1 = -(P1 - a.P1[c - pl]) / m->h3;
            face_fluxes(z1, z2, a.Xi1[c], a.ro1[c], a.Xi1[c - pl], a.ro1[c - pl], a.Xi1[c + pl], a.ro1[c + pl], &F1, &F2);
            s1 = fp32_dir(F1 * m->h3, F2 * m->h3, m->dt / (m->h3 * m->h3), 0);
            z2 = -(a.P2[c + pl] - P2) / m->h3;
            z1 = -(P2 - a.P2[c - pl]) / m->h3;
            face_fluxes(z1, z2, a.Xi2[c], a.ro2[c], a.Xi2[c - pl], a.ro2[c - pl], a.Xi2[c + pl], a.ro2[c + pl], &F1, &F2);
            s2 = fp32_dir(F1 * m->h3, F2 * m->h3, m->dt / (m->h3 * m->h3), 0);
          }
          x2 = -(a.P1[c + 1] - P1) / m->h1;
          x1 = -(P1 - a.P1[c - 1]) / m->h1;
          face_fluxes(x1, x2, a.Xi1[c], a.ro1[c], a.Xi1[c - 1], a.ro1[c - 1], a.Xi1[c + 1], a.ro1[c + 1], &F1, &F2);
          s1 = s1 + fp32_dir(F1 * m->h1, F2 * m->h1, m->dt / (m->h1 * m->h1), 0);
          y2 = -(a.P1[c + nx] - P1) / m->h2 + a.ro1[c] * m->g;
          y1 = -(P1 - a.P1[c - nx]) / m->h2 + a.ro1[c] * m->g;
          if (noflow_bottom && j == ny - 2) y2 = 0;
          face_fluxes(y1, y2, a.Xi1[c], a.ro1[c], a.Xi1[c - nx], a.ro1[c - nx], a.Xi1[c + nx], a.ro1[c + nx], &F1, &F2);
          s1 = s1 + fp32_dir(F1 * m->h2, F2 * m->h2, m->dt * m->kv / (m->h2 * m->h2), fy);
          x2 = -(a.P2[c + 1] - P2) / m->h1;
          x1 = -(P2 - a.P2[c - 1]) / m->h1;
          face_fluxes(x1, x2, a.Xi2[c], a.ro2[c], a.Xi2[c - 1], a.ro2[c - 1], a.Xi2[c + 1], a.ro2[c + 1], &F1, &F2);
          s2 = s2 + fp32_dir(F1 * m->h1, F2 * m->h1, m->dt / (m->h1 * m->h1), 0);
          y2 = -(a.P2[c + nx] - P2) / m->h2 + a.ro2[c] * m->g;
          y1 = -(P2 - a.P2[c - nx]) / m->h2 + a.ro2[c] * m->g;
          if (noflow_bottom && j == ny - 2) y2 = 0;
          face_fluxes(y1, y2, a.Xi2[c], a.ro2[c], a.Xi2[c - nx], a.ro2[c - nx], a.Xi2[c + nx], a.ro2[c + nx], &F1, &F2);
          if (ptop) {
            const double Fp = y1 >= 0 ? y1 * (-(a.Xi2[c - nx] * a.ro2[c - nx])) : y1 * (-(a.Xi2[c] * a.ro2[c]));
            pin = Fp * m->h2 * (m->dt * m->kv / (m->h2 * m->h2));
            F1 = 0.0;
          }
          s2 = s2 + fp32_dir(F1 * m->h2, F2 * m->h2, m->dt * m->kv / (m->h2 * m->h2), fy);
          /* the FP32 increments over phi (rounded), the patch inflow and the rate source exact */
          f1 = (double)(float)((double)s1 / phi);
          g1 = (double)(float)((double)s2 / phi);
          const double srcv = (src != 0.0 && j == 1 && orc_in_rate_patch(m, i, k)) ? (m->dt / phi) * src : 0.0;
          a.roS1_old[c] = roS1;
          a.roS2_old[c] = roS2;
          a.roS1[c] = roS1 + f1;
          a.roS2[c] = roS2 + g1 + pin / phi + srcv;
          continue;
        }
        double A1 = roS1 - (m->dt / phi) * (f1 + f2 + f3);
        double A2;
        if (src != 0.0 && j == 1 && orc_in_rate_patch(m, i, k))
          A2 = roS2 - (m->dt / phi) * ((g1 + g2 + g3) - src);
        else
          A2 = roS2 - (m->dt / phi) * (g1 + g2 + g3);
        a.roS1_old[c] = roS1;
        a.roS2_old[c] = roS2;
        a.roS1[c] = A1;
        a.roS2[c] = A2;
      }
}

/* a4: per-cell 2x2 Newton for (P1, S2) from the phase masses (cpu.cpp:293-320). */
void orc_newton(const gbf_model* m, const gbf_cells* cells, gbf_arrays a) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
#pragma omp parallel for schedule(static)
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz; k++) {
        if (!is_interior(m, i, j, k)) continue;
        size_t c = ORC_IDX(i, j, k);
        int md = media_of(cells, c);
        const double lam = m->lambda[md], swr = m->S_wr[md], pd = m->P_d[md];
        double S_e, P_k, AAA, F1, F2, PkS, F1P, F2P, F1S, F2S, det;
        for (int w = 1; w <= m->newton_iterations; w++) {
          double P1 = a.P1[c], S2 = a.S2[c];
          S_e = (1 - S2 - swr) / (1 - swr);
          P_k = pd * pow(S_e, (-1.) / lam);
          AAA = pow(S_e, (((-1.) / lam) - 1.));
          F1 = m->ro01 * (1. + (m->beta1) * (P1 - m->P_atm)) * (1. - S2) - a.roS1[c];
          F2 = m->ro02 * (1. + (m->beta2) * (P1 + P_k - m->P_atm)) * S2 - a.roS2[c];
          PkS = AAA * pd / (lam * (1 - swr));
          F1P = m->ro01 * (m->beta1) * (1 - S2);
          F2P = m->ro02 * (m->beta2) * S2;
          F1S = (-1) * m->ro01 * (1 + (m->beta1) * (P1 - m->P_atm));
          F2S = m->ro02 * (1 + (m->beta2) * (P1 + P_k - m->P_atm + (S2 * PkS)));
          det = F1P * F2S - F1S * F2P;
          double dP = (1 / det) * (F2S * F1 - F1S * F2);
          double dS = (1 / det) * (F1P * F2 - F2P * F1);
          a.P1[c] = P1 - dP;
          a.S2[c] = S2 - dS;
          if (m->newton_tol > 0 && fabs(dS) <= m->newton_tol && fabs(dP) <= m->newton_tol * fabs(a.P1[c]))
            break;
        }
      }
}

/* Hydrostatic profile of the initial state (main.cpp:114). */
static double p_hydrostatic(const gbf_model* m, int j) { return m->P_atm + j * m->ro01 * m->g * (m->h2); }

/* Border_S2 (cpu.cpp:323-363), in place, one cell. */
static void border_S2(const gbf_model* m, gbf_arrays a, int i, int j, int k) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  size_t c = ORC_IDX(i, j, k);
  const size_t pl = (size_t)nx * (size_t)ny;
  if ((i == 0) && (nx > 2)) { a.S2[c] = a.S2[c + 1]; return; }
  if ((i == nx - 1) && (nx > 2)) { a.S2[c] = a.S2[c - 1]; return; }
  if ((j == ny - 1) && (ny > 2)) { a.S2[c] = a.S2[c - nx]; return; }
  if ((j == 0) && (ny > 2)) {
    if (m->source_mode == GBF_SOURCE_DIRICHLET_PATCH && in_dirichlet_patch(m, i, k))
      a.S2[c] = m->S2_gr;
    else
      a.S2[c] = 0;
  }
  if ((k == 0) && (nz > 2)) { a.S2[c] = a.S2[c + pl]; return; }
  if ((k == nz - 1) && (nz > 2)) { a.S2[c] = a.S2[c - pl]; return; }
}

/* Border_P1 (cpu.cpp:366-403), in place, one cell. `ro1` is the start-of-step
   water density of a1; the bottom rule reads it at (i, 1, 0) (cpu.cpp:382). */
static void border_P1(const gbf_model* m, gbf_arrays a, int i, int j, int k) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  size_t c = ORC_IDX(i, j, k);
  const size_t pl = (size_t)nx * (size_t)ny;
  if (m->bc_mode == GBF_BC_HYDROSTATIC_SIDES &&
      ((i == 0) || (i == nx - 1) || (k == 0) || (k == nz - 1))) {
    a.P1[c] = p_hydrostatic(m, j);
    return;
  }
  if ((i == 0) && (nx > 2)) { a.P1[c] = a.P1[c + 1]; return; }
  if ((i == nx - 1) && (nx > 2)) { a.P1[c] = a.P1[c - 1]; return; }
  if ((j == ny - 1) && (ny > 2)) {
    a.P1[c] = a.P1[c - nx] + a.ro1[i + nx * 1] * m->g * (m->h2);
    return;
  }
  if ((j == 0) && (ny > 2)) { a.P1[c] = m->P_atm; return; }
  if ((k == 0) && (nz > 2)) { a.P1[c] = a.P1[c + pl]; return; }
  if ((k == nz - 1) && (nz > 2)) { a.P1[c] = a.P1[c - pl]; return; }
}

/* a5: one i->j->k sweep, Border_S2 then Border_P1 per cell (cpu.cpp:44-54). */
void orc_boundary(const gbf_model* m, gbf_arrays a) {
  for (int i = 0; i < m->nx; i++)
    for (int j = 0; j < m->ny; j++)
      for (int k = 0; k < m->nz; k++) {
        border_S2(m, a, i, j, k);
        border_P1(m, a, i, j, k);
      }
}

/* Phase masses sum(phi * roS_alpha * h1 h2 h3) over interior cells, taken
   after the mass update (no reference counterpart; used as the per-step
   mass-balance check). */
void orc_mass_totals(const gbf_model* m, const gbf_cells* cells, gbf_arrays a, double out[2]) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const double V = m->h1 * m->h2 * m->h3;
  double s1 = 0, s2 = 0;
  for (int k = 0; k < nz; k++)
    for (int j = 0; j < ny; j++)
      for (int i = 0; i < nx; i++) {
        if (!is_interior(m, i, j, k)) continue;
        size_t c = ORC_IDX(i, j, k);
        double phi = phi_of(m, cells, c, media_of(cells, c));
        s1 += phi * a.roS1[c] * V;
        s2 += phi * a.roS2[c] * V;
      }
  out[0] = s1;
  out[1] = s2;
}

/* One time step in the order of time_step_function (main.cpp:83-94); the
   exchange calls are the single-domain no-ops of no_communication.cpp. */
void orc_step(const gbf_model* m, const gbf_cells* cells, gbf_arrays a, int nsteps, double* mass_out) {
  for (int s = 0; s < nsteps; s++) {
    orc_props(m, cells, a);
    orc_velocity(m, a);
    orc_mass(m, cells, a);
    if (mass_out) orc_mass_totals(m, cells, a, mass_out + 2 * s);
    orc_newton(m, cells, a);
    orc_boundary(m, a);
  }
}

/* initial_data (main.cpp:97-138), single domain: S2 = S2_gr on the top patch
   (Dirichlet-patch mode; 0 in rate mode), hydrostatic P1, roS_old = 0. */
void orc_initial(const gbf_model* m, gbf_arrays a) {
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz; k++) {
        size_t c = ORC_IDX(i, j, k);
        if (m->source_mode == GBF_SOURCE_DIRICHLET_PATCH && (j == 0) && in_dirichlet_patch(m, i, k))
          a.S2[c] = m->S2_gr;
        else
          a.S2[c] = 0;
        a.P1[c] = p_hydrostatic(m, j);
        a.roS1_old[c] = 0;
        a.roS2_old[c] = 0;
      }
}
