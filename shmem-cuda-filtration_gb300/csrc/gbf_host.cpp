// gbf_host.cpp — status handling, model helpers and host-side validation.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include <atomic>

#include "gbf_internal.h"

namespace {
std::atomic<int> g_status{GBF_OK};
int g_num_sms = 0;
}  // namespace

int gbf_fail(int s, const char* where) {
  if (s != GBF_OK) {
    g_status.store(s);
    if (getenv("GBF_VERBOSE")) fprintf(stderr, "gbflow: %s (%s)\n", gbf_status_string(s), where ? where : "");
  }
  return s;
}

int gbf_cuda_check(cudaError_t e, const char* where) {
  if (e == cudaSuccess) return GBF_OK;
  // Same report as the reference's checkErrors (gpu.cu:7-27), but the error
  // is also kept as a status instead of being only printed.
  printf("CUDA Error: %s (at %s)\n", cudaGetErrorString(e), where ? where : "");
  fflush(stdout);
  return gbf_fail(e == cudaErrorMemoryAllocation ? GBF_ERR_NOMEM : GBF_ERR_CUDA, where);
}

int gbf_num_sms() {
  if (g_num_sms == 0) {
    int dev = 0, n = 0;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) == cudaSuccess && n > 0)
      g_num_sms = n;
    else
      g_num_sms = 152;
  }
  return g_num_sms;
}

cudaEvent_t gbf_timer_begin(GbfTimer* t, cudaStream_t st) {
  if (!t || !t->on) return nullptr;
  if (t->used == t->cap) {
    size_t ncap = t->cap ? 2 * t->cap : 64;
    cudaEvent_t* np = (cudaEvent_t*)realloc(t->pool, ncap * sizeof(cudaEvent_t));
    if (!np) return nullptr;
    for (size_t q = t->cap; q < ncap; q++) cudaEventCreate(&np[q]);
    t->pool = np;
    t->cap = ncap;
  }
  cudaEvent_t e = t->pool[t->used++];
  cudaEventRecord(e, st);
  return e;
}

void gbf_timer_end(GbfTimer* t, int kind, cudaEvent_t start, cudaStream_t st) {
  if (!t || !t->on || !start) return;
  cudaEvent_t e = gbf_timer_begin(t, st);
  if (!e) return;
  if (t->nrec == t->rcap) {
    size_t ncap = t->rcap ? 2 * t->rcap : 64;
    GbfTimer::Rec* nr = (GbfTimer::Rec*)realloc(t->recs, ncap * sizeof(GbfTimer::Rec));
    if (!nr) return;
    t->recs = nr;
    t->rcap = ncap;
  }
  t->recs[t->nrec++] = {kind, start, e};
}

int gbf_timer_collect(GbfTimer* t, double* ms, int* launches, int nkinds) {
  for (int k = 0; k < nkinds; k++) { ms[k] = 0; launches[k] = 0; }
  if (!t) return GBF_OK;
  for (size_t r = 0; r < t->nrec; r++) {
    float x = 0;
    cudaEventSynchronize(t->recs[r].b);
    if (cudaEventElapsedTime(&x, t->recs[r].a, t->recs[r].b) == cudaSuccess && t->recs[r].kind < nkinds) {
      ms[t->recs[r].kind] += x;
      launches[t->recs[r].kind]++;
    }
  }
  t->nrec = 0;
  t->used = 0;
  return GBF_OK;
}

void gbf_timer_free(GbfTimer* t) {
  if (!t) return;
  for (size_t q = 0; q < t->cap; q++) cudaEventDestroy(t->pool[q]);
  free(t->pool);
  free(t->recs);
  t->pool = nullptr;
  t->recs = nullptr;
  t->cap = t->used = t->nrec = t->rcap = 0;
}

// Page-locked host arrays are read and written in place by the conversion
// kernels (over NVLink-C2C) instead of being staged by copy-engine copies.
static std::atomic<int> g_host_direct{1};

const void* gbf_mapped_host(const void* p) {
  if (!p || !g_host_direct.load()) return nullptr;
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();  // unregistered memory on older runtimes: not an error here
    return nullptr;
  }
  return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

extern "C" {

const char* gbf_kernel_name(int kind) {
  static const char* names[GBF_K_COUNT] = {"f64_props", "f64_flux_newton", "f64_boundary", "mass_tail",
                                           "split_step", "split_boundary", "ensemble_step", "ensemble_boundary",
                                           "ensemble_f64_props", "ensemble_f64_flux_newton"};
  return (kind >= 0 && kind < GBF_K_COUNT) ? names[kind] : "";
}
int gbf_kernel_kinds(void) { return GBF_K_COUNT; }

int gbf_last_status(void) { return g_status.load(); }
void gbf_clear_status(void) { g_status.store(GBF_OK); }

int gbf_set_host_direct(int on) {
  if (on < 0) return g_host_direct.load();
  return g_host_direct.exchange(on ? 1 : 0);
}

const char* gbf_status_string(int s) {
  switch (s) {
    case GBF_OK: return "ok";
    case GBF_ERR_ARG: return "invalid argument";
    case GBF_ERR_CUDA: return "CUDA error";
    case GBF_ERR_NOMEM: return "out of device memory";
    case GBF_ERR_NONFINITE: return "non-finite pressure or saturation";
    case GBF_ERR_UNSTABLE: return "time step above the explicit stability bound";
    case GBF_ERR_TIMEOUT: return "device-side wait timed out";
    case GBF_ERR_STATE: return "call out of order";
    default: return "unknown status";
  }
}

const char* gbf_version(void) { return "gbflow 0.1 (sm_103a)"; }

size_t gbf_abi_sizeof(int which) {
  switch (which) {
    case 0: return sizeof(gbf_model);
    case 1: return sizeof(gbf_cells);
    case 2: return sizeof(gbf_arrays);
    case 3: return sizeof(gbf_run_defines);
    default: return 0;
  }
}

// The reference's compile-time constants (defines.h:6-26) and the values of
// its defines.ini; NX/Ny/Nz and dt from the arguments.
void gbf_model_reference(gbf_model* m, int nx, int ny, int nz, double dt) {
  if (!m) return;
  gbf_model r = {};
  r.nx = nx; r.ny = ny; r.nz = nz;
  r.h1 = 0.02045; r.h2 = 0.01969; r.h3 = 0.01969; r.dt = dt;
  r.K[0] = 6.64e-11; r.K[1] = 7.15e-12;
  r.lambda[0] = 2.7; r.lambda[1] = 2.0;
  r.S_wr[0] = 0.09; r.S_wr[1] = 0.12;
  r.m[0] = 0.4; r.m[1] = 0.39;
  r.P_d[0] = 755; r.P_d[1] = 2060;
  r.beta1 = 1.0e-4; r.beta2 = 1.0e-8;
  r.mu1 = 0.001; r.mu2 = 0.0009; r.ro01 = 1000; r.ro02 = 1460;
  r.S2_gr = 0.4; r.P_atm = 100000; r.g = 9.8;
  r.source = 3; r.newton_iterations = 7;
  r.source_mode = GBF_SOURCE_DIRICHLET_PATCH; r.rate_cells = 0; r.rate = 0;
  r.bc_mode = GBF_BC_REFERENCE; r.kv = 1.0; r.newton_tol = 0;
  *m = r;
}

int gbf_model_validate(const gbf_model* m, const gbf_cells* cells, int check_dt) {
  if (!m) return gbf_fail(GBF_ERR_ARG, "model is NULL");
  if (m->nx < 3 || m->ny < 3 || m->nz < 3) return gbf_fail(GBF_ERR_ARG, "grid dimensions must be >= 3");
  // kernels index one grid with 32-bit offsets
  if ((double)m->nx * m->ny * m->nz >= 2147483648.0) return gbf_fail(GBF_ERR_ARG, "grid holds 2^31 cells or more");
  if (!(m->h1 > 0 && m->h2 > 0 && m->h3 > 0 && m->dt > 0)) return gbf_fail(GBF_ERR_ARG, "h and dt must be > 0");
  if (!(m->mu1 > 0 && m->mu2 > 0 && m->ro01 > 0 && m->ro02 > 0)) return gbf_fail(GBF_ERR_ARG, "fluid constants");
  if (m->newton_iterations < 1 || m->newton_iterations > 64) return gbf_fail(GBF_ERR_ARG, "newton_iterations");
  if (!(m->kv > 0)) return gbf_fail(GBF_ERR_ARG, "kv must be > 0");
  for (int md = 0; md < 2; md++) {
    if (!(m->lambda[md] > 0) || !(m->S_wr[md] >= 0 && m->S_wr[md] < 1) || !(m->m[md] > 0) || !(m->P_d[md] >= 0))
      return gbf_fail(GBF_ERR_ARG, "media table");
    // The Dirichlet patch saturation must leave S_e > 0 (Brooks-Corey P_k finite).
    if (m->source_mode == GBF_SOURCE_DIRICHLET_PATCH && !(1.0 - m->S2_gr - m->S_wr[md] > 0))
      return gbf_fail(GBF_ERR_ARG, "S2_gr leaves no mobile water (S_e <= 0)");
  }
  if (m->source_mode == GBF_SOURCE_RATE) {
    if (m->rate_cells < 1 || m->rate_cells > m->nx - 2 || m->rate_cells > m->nz - 2 || !(m->rate >= 0))
      return gbf_fail(GBF_ERR_ARG, "rate patch");
  }
  const size_t n = (size_t)m->nx * m->ny * m->nz;
  if (cells) {
    for (size_t c = 0; c < n; c++) {
      if (cells->media && (cells->media[c] < 0 || cells->media[c] > 1)) return gbf_fail(GBF_ERR_ARG, "media index");
      if (cells->K && !(cells->K[c] > 0 && isfinite(cells->K[c]))) return gbf_fail(GBF_ERR_ARG, "K must be > 0");
      if (cells->phi && !(cells->phi[c] > 0 && cells->phi[c] <= 1)) return gbf_fail(GBF_ERR_ARG, "phi in (0, 1]");
    }
  }
  if (check_dt) {
    double dts = gbf_stable_dt(m, cells, 1.0);
    if (m->dt > dts) return gbf_fail(GBF_ERR_UNSTABLE, "dt above the stability bound");
  }
  return GBF_OK;
}

}  // extern "C"
