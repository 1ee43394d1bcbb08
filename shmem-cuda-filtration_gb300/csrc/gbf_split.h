// gbf_split.h — split-precision (FP32 state, FP64 or FP32-pair masses)
// launchers and the constants of its kernels.
#pragma once

#include "gbf_domain.h"

// Model constants of the split kernels, derived once on the host. FP32 for
// the FP32 arithmetic; FP64 and FP32-pair copies for the wide residual.
struct GbfSplitConsts {
  int nx, ny, nz;
  int noflow_bottom;  // GBF_BC_HYDROSTATIC_SIDES: no-flow bottom face and hydrostatic P on the i and k sides
  int ri0, rk0, rn;  // the source's cells on the j = 1 layer: the rate injection's or those under the Dirichlet patch (rn = 0: none)
  float H;  // rho01 g h2: hydrostatic pressure step per cell (main.cpp:114)
  // Face potentials are kept as pressure differences (times h): their
  // gravity terms g rho01 beta1 h2, g rho02 beta2 h2, g (rho02 - rho01) h2,
  // and the flux-difference weights dt / h1^2, dt kv / h2^2, dt / h3^2 that
  // turn the upwinded face products into mass increments (times 1 / phi).
  float gh1, gh2, ghd;
  float wx, wy, wz;
  float cfl1, cfl2;  // 1 / rho0 of each phase: face mass flux -> volumetric flux (CFL numbers)
  float ro01, ro02, beta1, beta2, bmax;  // bmax = max(beta1, beta2)
  float nmr1, nmr2;      // -rho01 / mu1, -rho02 / mu2
  float ro01b1, ro02b2;  // rho01 beta1, rho02 beta2
  float ro01b1_lo, ro02b2_lo;  // their FP64 values' remainders (pairs; the residual-correction step)
  float K[2], m[2], e1[2], e2[2], m_inv_lam[2], inv_lam_1mswr[2], P_d[2];
  float se_b[2];  // S_e = 1 + se_b S = (1 - S_wr - S) / (1 - S_wr)
  double H_d, beta1_d, beta2_d, ro01_d, ro02_d, dtsrc_d, V;
  float2 H_df, beta1_df, beta2_df, ro01_df, ro02_df, dtsrc_df;
  // media-table porosity and dt*src/phi in wide precision: the table values
  // (e.g. 0.4) are not FP32 numbers, and the phase masses must not inherit
  // the FP32 rounding of phi
  double m_d[2], dtsrc_m_d[2];
  float2 m_df[2], dtsrc_m_df[2];
  double ro01b1_d, ro02b2_d;  // rho01 beta1, rho02 beta2 (the defect form's row densities)
};
GbfSplitConsts gbf_split_consts(const gbf_model& m);

// The reference's Dirichlet patch (GBF_SOURCE_DIRICHLET_PATCH): top-face cells
// i in [i0, i0 + n), k in [k0, k0 + n) that hold S2_gr and P_atm (cpu.cpp:346).
// The split forms take the DNAPL inflow of the j = 1 cells below them in FP64
// from the step's pre-pass (gbf_split_patch_cell); its constants, apart from
// the tiles' GbfSplitConsts (where ri0, rk0, rn then mark the same cells).
// n = 0: no patch.
struct GbfPatchConsts {
  int i0, k0, n;
  double S2, nmr2, gh2, wy;     // S2_gr, -rho02 / mu2, g h2, dt kv / h2^2
  double K[2], se_b[2], e2[2];  // media table: K, -1 / (1 - S_wr), (2 + lambda) / lambda
};
GbfPatchConsts gbf_patch_consts(const gbf_model& m);

// A row's constants for the conversions between the FP64 state and the split
// state: the hydrostatic pressure P_hs(j) and the defect forms' row densities
// c1(j), c2(j) (gbf_row_const). Grids keep a table of them, one entry per row
// j, filled once on the device, so that converting a whole grid does the FP64
// row arithmetic once per row instead of once per cell.
struct GbfRowConst {
  double phs;
  float c1, c2;
};
// Fill rows[0, ny) for the model (stream-ordered on st).
int gbf_split_fill_rows(const gbf_model& m, GbfRowConst* rows, cudaStream_t st);

// How the split forms hold the per-cell phase masses M1, M2 (gbf_split_tile.cuh):
// kMassDF FP32 pairs; kMassDefect FP32 defects over the mass of the FP32
// state at the row's hydrostatic density (4 bytes); kMassDefectDF the same
// defects as FP32 pairs (8 bytes; GBF_PREC_SPLIT: masses at least as precise
// as FP64). kMassF64 (the masses themselves in FP64) is the wide
// arithmetic's FP64 flavour, not a form.
enum { kMassF64 = 0, kMassDF = 1, kMassDefect = 2, kMassDefectDF = 3 };
__host__ __device__ constexpr bool gbf_is_defect(int mr) { return mr == kMassDefect || mr == kMassDefectDF; }
__host__ __device__ inline int gbf_mass_rep(int precision) {
  return precision == GBF_PREC_SPLIT_DEFECT ? kMassDefect : precision == GBF_PREC_SPLIT_DF ? kMassDF : kMassDefectDF;
}
__host__ __device__ inline int gbf_mass_bytes(int mr) { return mr == kMassDefect ? 4 : 8; }

// Arrays of one grid's split-precision step.
struct GbfSplitGrid {
  const float* dP;  // current state
  const float* S;
  float* dPn;       // next state
  float* Sn;
  const float* K;   // NULL: media table
  const float* phi;
  const int* media;
  double* M1;       // FP64, float2 pairs in the same 8 bytes, or FP32 defects (4 bytes)
  double* M2;
  double* mass_partials;  // NULL: no phase-mass sums
  unsigned* status;
  float* cfl_out;  // NULL: no CFL numbers; else the step's [2] slot (max-combined with atomicMax)
  // Dirichlet patch (the PATCH tiles): the FP64 DNAPL inflow of the j = 1
  // cells under it, (i - ri0) + rn (k - rk0), as FP32 pairs, written by the
  // step's pre-pass (gbf_split_patch_cell); NULL without a patch
  float2* patch_in;
};

int gbf_split_alloc(gbf_domain* d);
int gbf_split_upload(gbf_domain* d, const double* P1, const double* S2, cudaMemcpyKind kind);
int gbf_split_step(gbf_domain* d);
int gbf_split_download(gbf_domain* d, int field, double* host);
int gbf_split_launches_per_step(gbf_domain* d);
// upload + one step + download from and to host FP64 arrays, pipelined over
// slabs of planes (gbf_domain_advance_host; grids without a Dirichlet patch,
// large enough for two slabs of about 1M cells: gbf_split_pipelined).
int gbf_split_advance_host(gbf_domain* d, const double* P_in, const double* S_in, double* P_out, double* S_out);
bool gbf_split_pipelined(const gbf_model& m);
// FP64 (P, S) of every cell from a split state (device arrays; either output
// may be NULL; rows: the grid's row table, or NULL to form each row's values
// per cell).
int gbf_split_state_to_f64(const gbf_model& m, const GbfRowConst* rows, const float* dPf, const float* Sf, double* P,
                           double* S, cudaStream_t st);
// FP32 state and wide masses of one grid from FP64 device arrays (rows as above).
int gbf_split_init_state(const gbf_model& m, const GbfRowConst* rows, const double* P_dev, const double* S_dev,
                         float* dPf, float* Sf, double* M1, double* M2, int mr, cudaStream_t st);
// V sum over interior cells of c1(j) phi (the defect form's water mass of a
// fully water-saturated grid at the row densities): the part of the phase-1
// mass the tiles' sums leave out. Written to *k1v_host; 0 for other forms.
int gbf_defect_k1(const gbf_model& m, const float* phi_dev, const int* media_dev, double* k1v_host,
                  cudaStream_t st);
struct GbfTmaSet;
// `maps` (device memory; boxes of the x-pair tile) selects the x-pair TMA
// tile for state buffer `buf`; without it the plain-load 32x8 tile runs.
int gbf_split_launch_domain(const gbf_model& m, const GbfSplitConsts& C, const GbfSplitGrid& G, int mr,
                            double* mass_out, cudaStream_t st, GbfTimer* tm, const GbfTmaSet* maps, int buf,
                            double k1v);
