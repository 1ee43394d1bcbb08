// gbf_domain.h — internal definition of gbf_domain and the kernel launchers
// shared by the FP64, split-precision and drop-in code (not installed).
#pragma once

#include <vector>

#include "gbf_internal.h"

// Per-media constants derived once on the host (divisions hoisted out of
// the kernels).
struct GbfDerived {
  double inv_1mswr[2];      // 1 / (1 - S_wr)
  double e1[2], e2[2];      // Brooks-Corey exponents (2 + 3 lambda)/lambda, (2 + lambda)/lambda
  double m_inv_lam[2];      // -1 / lambda
  double inv_lam_1mswr[2];  // 1 / (lambda (1 - S_wr))
  double neg_inv_mu1, neg_inv_mu2;
  double inv_h1, inv_h2, inv_h3;
  double src;  // rate-mode source per unit volume [kg/(m^3 s)], 0 otherwise
  double V;    // cell volume
};
GbfDerived gbf_derive(const gbf_model& m);

// Props-pass output flags.
enum { GBF_PF_WRITE_XI_P2 = 1, GBF_PF_WRITE_U = 2 };

struct GbfF64Step {
  const double* P;  // current state (read)
  const double* S;
  double* Pn;       // next state (interior from the flux pass, faces from the boundary pass)
  double* Sn;
  double *L1, *L2;  // Xi * ro per phase (upwinded mobility x density)
  double *ro1, *ro2, *lnSe;
  double *Xi1, *Xi2, *P2;                     // GBF_PF_WRITE_XI_P2
  double *u1x, *u1y, *u1z, *u2x, *u2y, *u2z;  // GBF_PF_WRITE_U
  double *roS1, *roS2, *roS1_old, *roS2_old;  // optional (NULL: not written)
  double* mass_partials;                      // optional, 2 per block of the flux pass
  unsigned* status;                           // device status bits
};

// Device status bits (OR-ed by kernels, read by gbf_domain_status).
enum { GBF_DEV_NONFINITE = 1u, GBF_DEV_TIMEOUT = 2u };

// FP64 launchers (gbf_f64.cu).
unsigned gbf_f64_flux_grid(const gbf_model& m);
int gbf_f64_launch_step(const gbf_model& m, const GbfDerived& d, const gbf_cells& cells, const GbfF64Step& s,
                        int props_flags, double* mass_out, cudaStream_t st, GbfTimer* tm);

struct gbf_domain {
  gbf_model m;
  GbfDerived d;
  int precision = GBF_PREC_F64;
  int out_flags = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  // cells (device)
  gbf_cells cells = {nullptr, nullptr, nullptr};
  int* own_media = nullptr;
  float *own_K = nullptr, *own_phi = nullptr;
  // FP64 state and props
  double *P[2] = {nullptr, nullptr}, *S[2] = {nullptr, nullptr};
  int cur = 0;
  double *L1 = nullptr, *L2 = nullptr, *ro1 = nullptr, *ro2 = nullptr, *lnSe = nullptr;
  gbf_arrays outs = {};  // optional reference arrays (velocity, masses, Xi, P2)
  // split-precision state (gbf_split.cu)
  float *Pf[2] = {nullptr, nullptr}, *Sf[2] = {nullptr, nullptr};
  double *M1 = nullptr, *M2 = nullptr;
  double* split_partials = nullptr;
  float2* split_patch = nullptr;  // the Dirichlet patch's FP64 inflow (split forms; NULL without a patch)
  struct GbfRowConst* split_rows = nullptr;  // the split state conversions' row table (ny entries)
  // host-resident pipeline of the split forms (gbf_domain_advance_host): copy
  // streams, their events, an FP64 staging copy of (P, S) (allocated on first use)
  cudaStream_t pipe_in = nullptr, pipe_out = nullptr;
  std::vector<cudaEvent_t> pipe_ev;
  double* pipe_stage = nullptr;
  double defect_k1v = 0.0;  // defect form: V sum of c1(j) phi over interior cells (gbf_defect_k1)
  void* tma = nullptr;  // device GbfTmaSet of the split state (NULL: plain loads)
  // mass tracking
  double* mass_partials = nullptr;
  double* mass_hist = nullptr;
  float* cfl_hist = nullptr;  // [mass_cap][2] (GBF_OUT_CFL)
  int mass_cap = 0;
  long long mass_count = 0;
  unsigned* status = nullptr;
  long long steps = 0;
  bool uploaded = false;
  // drop-in attachment: state arrays belong to the caller
  bool borrowed = false;
  gbf_arrays caller = {};
  int pending = 0;
  double* bscratch = nullptr;  // boundary gather scratch of the one-kernel-per-stage fallback
  bool lazy_dirty = false;     // drop-in: derived arrays not yet materialised for the last fused step
  // drop-in split mode (a split-precision domain behind the caller's FP64
  // arrays): split_stale, the caller's P1/S2 were written since the split
  // state was formed from them; caller_stale, the split state is ahead of the
  // caller's P1/S2 (written back when the host reads them)
  bool split_stale = true, caller_stale = false;
  std::vector<void*> owned;  // every cudaMalloc of this domain
  GbfTimer timer;
};

int gbf_domain_alloc(gbf_domain* d, void** p, size_t bytes);

// roS1_old, roS2_old of interior cells from an FP64 state (P, S) or, with P
// and S NULL, from a split state (dPf, Sf); boundary cells 0 (gbf_eager.cu).
int gbf_roS_old_launch(const gbf_model& m, const double* P, const double* S, const float* dPf, const float* Sf,
                       double* o1, double* o2, cudaStream_t st);

// Drop-in helpers (gbf_domain.cu).
// precision: GBF_PREC_F64 (the fused mode) or a split form (the split mode).
int gbf_domain_attach_dropin(const gbf_model* m, gbf_arrays caller, gbf_cells cells, int precision, gbf_domain** out);
int gbf_dropin_defer(gbf_domain* d, const gbf_model& m, int stage);
int gbf_dropin_flush(gbf_domain* d);
void gbf_domain_detach_dropin(gbf_domain* d);
int gbf_dropin_materialize(gbf_domain* d);
bool gbf_dropin_is_derived(const gbf_domain* d, const double* p);
// Split mode: the caller's P1 and S2 from the split state when it is ahead of
// them (before the host reads them or an eager stage runs on them), and the
// note that the host wrote one of them (the split state is formed anew).
int gbf_dropin_writeback(gbf_domain* d);
void gbf_dropin_host_wrote(gbf_domain* d, const double* dev);
// The host rewrote the media array `dev`, which the domain reads in place:
// the split defect form's porosity sum over the rows (a constant of its mass
// sums, taken from the media at creation) is taken again.
int gbf_dropin_media_wrote(gbf_domain* d, const int* dev);
