// gbf_eager.cu — one FP64 kernel per hot-path function of the reference.
//
// These are the kernels behind the drop-in's default (eager) mode: each
// reference function call launches its own kernel and writes the reference's
// arrays, so any caller of the defines.h function set sees exactly the
// reference's intermediate state. Semantics follow the reference CPU path
// (cpu.cpp), which is the oracle:
//   * a 3-D iteration space covered by a flat grid-stride loop (the reference
//     GPU kernels' blockIdx.y / BlockNY split, gpu.cu:61-62, leaves cells
//     untouched whenever ceil(Ny/4) != 4; this mapping has no such gap);
//   * model.newton_iterations Newton iterations (7 in the reference CPU path,
//     defines.h:15; the reference GPU kernel runs one, gpu.cu:342-374);
//   * boundary values of the CPU's in-place i->j->k sweep (cpu.cpp:44-54),
//     computed race-free in two kernels (gather to scratch, then scatter).
//
// This translation unit is compiled with -fmad=false so that every
// multiply-add rounds like the oracle's; only pow() may differ in the last
// bit between CUDA and the host libm.
#include <math.h>

#include <mutex>

#include <cuda.h>
#include <cudaTypedefs.h>

#include "gbf_internal.h"

namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int media_at(const gbf_cells& c, size_t idx) { return c.media ? c.media[idx] : 0; }
__device__ __forceinline__ double K_at(const gbf_model& m, const gbf_cells& c, size_t idx, int md) {
  return c.K ? (double)c.K[idx] : m.K[md];
}
__device__ __forceinline__ double phi_at(const gbf_model& m, const gbf_cells& c, size_t idx, int md) {
  return c.phi ? (double)c.phi[idx] : m.m[md];
}

// a1 (cpu.cpp:57-74): every cell.
__global__ void __launch_bounds__(kThreads) k_props(const gbf_model m, gbf_arrays a, gbf_cells cells) {
  const GbfGeo g = gbf_geo(m);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.n; c += (size_t)gridDim.x * blockDim.x) {
    int md = media_at(cells, c);
    double K = K_at(m, cells, c, md);
    double S2 = a.S2[c], P1 = a.P1[c];
    double S_e = (1. - S2 - m.S_wr[md]) / (1. - m.S_wr[md]);
    double k1 = pow(S_e, (2. + 3. * m.lambda[md]) / m.lambda[md]);
    double k2 = (1. - S_e) * (1. - S_e) * (1 - pow(S_e, (2. + m.lambda[md]) / m.lambda[md]));
    double P2 = P1 + 0.0;
    a.P2[c] = P2;
    a.Xi1[c] = -1. * K * k1 / m.mu1;
    a.Xi2[c] = -1. * K * k2 / m.mu2;
    a.ro1[c] = m.ro01 * (1. + (m.beta1) * (P1 - m.P_atm));
    a.ro2[c] = m.ro02 * (1. + (m.beta2) * (P2 - m.P_atm));
  }
}

// a2 (cpu.cpp:77-160): every cell; one-sided differences on the faces.
__global__ void __launch_bounds__(kThreads) k_velocity(const gbf_model m, gbf_arrays a) {
  const GbfGeo g = gbf_geo(m);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.n; c += (size_t)gridDim.x * blockDim.x) {
    int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / g.pl);
    double Xi1 = a.Xi1[c], Xi2 = a.Xi2[c];
    if (i == 0) {
      a.u1x[c] = Xi1 * (a.P1[c + 1] - a.P1[c]) / (m.h1);
      a.u2x[c] = Xi2 * (a.P2[c + 1] - a.P2[c]) / (m.h1);
    } else if (i == g.nx - 1) {
      a.u1x[c] = Xi1 * (a.P1[c] - a.P1[c - 1]) / (m.h1);
      a.u2x[c] = Xi2 * (a.P2[c] - a.P2[c - 1]) / (m.h1);
    } else {
      a.u1x[c] = Xi1 * ((a.P1[c + 1] - a.P1[c - 1]) / (2. * (m.h1)));
      a.u2x[c] = Xi2 * ((a.P2[c + 1] - a.P2[c - 1]) / (2. * (m.h1)));
    }
    const size_t up = c - g.nx, dn = c + g.nx;
    const double kX1 = m.kv * Xi1, kX2 = m.kv * Xi2;
    if (j == 0) {
      a.u1y[c] = kX1 * ((a.P1[dn] - a.P1[c]) / (m.h2) - a.ro1[c] * m.g);
      a.u2y[c] = kX2 * ((a.P2[dn] - a.P2[c]) / (m.h2) - a.ro2[c] * m.g);
    } else if (j == g.ny - 1) {
      a.u1y[c] = kX1 * ((a.P1[c] - a.P1[up]) / (m.h2) - a.ro1[c] * m.g);
      a.u2y[c] = kX2 * ((a.P2[c] - a.P2[up]) / (m.h2) - a.ro2[c] * m.g);
    } else {
      a.u1y[c] = kX1 * ((a.P1[dn] - a.P1[up]) / (2. * (m.h2)) - a.ro1[c] * m.g);
      a.u2y[c] = kX2 * ((a.P2[dn] - a.P2[up]) / (2. * (m.h2)) - a.ro2[c] * m.g);
    }
    if (k == 0) {
      a.u1z[c] = Xi1 * (a.P1[c + g.pl] - a.P1[c]) / (m.h3);
      a.u2z[c] = Xi2 * (a.P2[c + g.pl] - a.P2[c]) / (m.h3);
    } else if (k == g.nz - 1) {
      a.u1z[c] = Xi1 * (a.P1[c] - a.P1[c - g.pl]) / (m.h3);
      a.u2z[c] = Xi2 * (a.P2[c] - a.P2[c - g.pl]) / (m.h3);
    } else {
      a.u1z[c] = Xi1 * ((a.P1[c + g.pl] - a.P1[c - g.pl]) / (2. * (m.h3)));
      a.u2z[c] = Xi2 * ((a.P2[c + g.pl] - a.P2[c - g.pl]) / (2. * (m.h3)));
    }
  }
}

// Donor-cell divergence of one direction (cpu.cpp:260-262), reference order.
__device__ __forceinline__ double upwind_div(double x1, double x2, double Xc, double rc, double Xm, double rm,
                                             double Xp, double rp, double h) {
  return (((x2 + fabs(x2)) / 2.0 - (x1 - fabs(x1)) / 2.0) * (-1) * Xc * rc -
          (x1 + fabs(x1)) / 2.0 * (-1) * Xm * rm +
          (x2 - fabs(x2)) / 2.0 * (-1) * Xp * rp) / h;
}

__device__ __forceinline__ void interior_cell(const GbfGeo& g, size_t t, int& i, int& j, int& k) {
  size_t ix = (size_t)g.nx - 2, iy = (size_t)g.ny - 2;
  i = 1 + (int)(t % ix);
  j = 1 + (int)((t / ix) % iy);
  k = 1 + (int)(t / (ix * iy));
}

// a3 (cpu.cpp:218-291): interior cells.
__global__ void __launch_bounds__(kThreads) k_mass(const gbf_model m, gbf_arrays a, gbf_cells cells) {
  const GbfGeo g = gbf_geo(m);
  const size_t nint = (size_t)(g.nx - 2) * (g.ny - 2) * (g.nz - 2);
  const bool noflow_bottom = (m.bc_mode == GBF_BC_HYDROSTATIC_SIDES);
  const double src = (m.source_mode == GBF_SOURCE_RATE && m.rate_cells > 0)
                         ? m.rate / (double)(m.rate_cells * m.rate_cells) / (m.h1 * m.h2 * m.h3)
                         : 0.0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nint; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    interior_cell(g, t, i, j, k);
    const size_t c = gbf_idx(g, i, j, k), pl = g.pl, nx = g.nx;
    int md = media_at(cells, c);
    double phi = phi_at(m, cells, c, md);
    double roS1 = a.ro1[c] * (1 - a.S2[c]);
    double roS2 = a.ro2[c] * a.S2[c];
    double P1 = a.P1[c], P2 = a.P2[c];
    double x1, x2, y1, y2, z1, z2;
    z2 = -(a.P1[c + pl] - P1) / m.h3;
    z1 = -(P1 - a.P1[c - pl]) / m.h3;
    double f3 = upwind_div(z1, z2, a.Xi1[c], a.ro1[c], a.Xi1[c - pl], a.ro1[c - pl], a.Xi1[c + pl], a.ro1[c + pl], m.h3);
    z2 = -(a.P2[c + pl] - P2) / m.h3;
    z1 = -(P2 - a.P2[c - pl]) / m.h3;
    double g3 = upwind_div(z1, z2, a.Xi2[c], a.ro2[c], a.Xi2[c - pl], a.ro2[c - pl], a.Xi2[c + pl], a.ro2[c + pl], m.h3);
    x2 = -(a.P1[c + 1] - P1) / m.h1;
    x1 = -(P1 - a.P1[c - 1]) / m.h1;
    y2 = -(a.P1[c + nx] - P1) / m.h2 + a.ro1[c] * m.g;
    y1 = -(P1 - a.P1[c - nx]) / m.h2 + a.ro1[c] * m.g;
    if (noflow_bottom && j == g.ny - 2) y2 = 0;
    double f1 = upwind_div(x1, x2, a.Xi1[c], a.ro1[c], a.Xi1[c - 1], a.ro1[c - 1], a.Xi1[c + 1], a.ro1[c + 1], m.h1);
    double f2 = m.kv * upwind_div(y1, y2, a.Xi1[c], a.ro1[c], a.Xi1[c - nx], a.ro1[c - nx], a.Xi1[c + nx], a.ro1[c + nx], m.h2);
    x2 = -(a.P2[c + 1] - P2) / m.h1;
    x1 = -(P2 - a.P2[c - 1]) / m.h1;
    y2 = -(a.P2[c + nx] - P2) / m.h2 + a.ro2[c] * m.g;
    y1 = -(P2 - a.P2[c - nx]) / m.h2 + a.ro2[c] * m.g;
    if (noflow_bottom && j == g.ny - 2) y2 = 0;
    double g1 = upwind_div(x1, x2, a.Xi2[c], a.ro2[c], a.Xi2[c - 1], a.ro2[c - 1], a.Xi2[c + 1], a.ro2[c + 1], m.h1);
    double g2 = m.kv * upwind_div(y1, y2, a.Xi2[c], a.ro2[c], a.Xi2[c - nx], a.ro2[c - nx], a.Xi2[c + nx], a.ro2[c + nx], m.h2);
    double A1 = roS1 - (m.dt / phi) * (f1 + f2 + f3);
    double A2 = (src != 0.0 && j == 1 && gbf_in_rate_patch(m, i, k))
                    ? roS2 - (m.dt / phi) * ((g1 + g2 + g3) - src)
                    : roS2 - (m.dt / phi) * (g1 + g2 + g3);
    a.roS1_old[c] = roS1;
    a.roS2_old[c] = roS2;
    a.roS1[c] = A1;
    a.roS2[c] = A2;
  }
}

// a4 (cpu.cpp:293-320): interior cells, in place.
__global__ void __launch_bounds__(kThreads) k_newton(const gbf_model m, gbf_arrays a, gbf_cells cells) {
  const GbfGeo g = gbf_geo(m);
  const size_t nint = (size_t)(g.nx - 2) * (g.ny - 2) * (g.nz - 2);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nint; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    interior_cell(g, t, i, j, k);
    const size_t c = gbf_idx(g, i, j, k);
    int md = media_at(cells, c);
    const double lam = m.lambda[md], swr = m.S_wr[md], pd = m.P_d[md];
    const double roS1 = a.roS1[c], roS2 = a.roS2[c];
    double P1 = a.P1[c], S2 = a.S2[c];
    for (int w = 1; w <= m.newton_iterations; w++) {
      double S_e = (1 - S2 - swr) / (1 - swr);
      double P_k = pd * pow(S_e, (-1.) / lam);
      double AAA = pow(S_e, (((-1.) / lam) - 1.));
      double F1 = m.ro01 * (1. + (m.beta1) * (P1 - m.P_atm)) * (1. - S2) - roS1;
      double F2 = m.ro02 * (1. + (m.beta2) * (P1 + P_k - m.P_atm)) * S2 - roS2;
      double PkS = AAA * pd / (lam * (1 - swr));
      double F1P = m.ro01 * (m.beta1) * (1 - S2);
      double F2P = m.ro02 * (m.beta2) * S2;
      double F1S = (-1) * m.ro01 * (1 + (m.beta1) * (P1 - m.P_atm));
      double F2S = m.ro02 * (1 + (m.beta2) * (P1 + P_k - m.P_atm + (S2 * PkS)));
      double det = F1P * F2S - F1S * F2P;
      double dP = (1 / det) * (F2S * F1 - F1S * F2);
      double dS = (1 / det) * (F1P * F2 - F2P * F1);
      P1 = P1 - dP;
      S2 = S2 - dS;
      if (m.newton_tol > 0 && fabs(dS) <= m.newton_tol && fabs(dP) <= m.newton_tol * fabs(P1)) break;
    }
    a.P1[c] = P1;
    a.S2[c] = S2;
  }
}

// a5, pass 1: the value the reference's sweep leaves at every boundary cell,
// into scratch[0 .. nb) (S2) and scratch[nb .. 2nb) (P1). Reads only.
__global__ void __launch_bounds__(kThreads) k_boundary_gather(const gbf_model m, gbf_arrays a, double* scratch) {
  const GbfGeo g = gbf_geo(m);
  const size_t nb = gbf_boundary_count(g);
  const double* ro1 = a.ro1;
  auto ro1_top = [ro1, &g](int i) { return ro1[(size_t)i + (size_t)g.nx]; };
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nb; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    gbf_boundary_cell(g, t, i, j, k);
    scratch[t] = gbf_sweep_S<double>(m, g, a.S2, a.S2, i, j, k);
    scratch[nb + t] = gbf_sweep_P<double>(m, g, a.P1, a.P1, i, j, k, ro1_top);
  }
}

// a5, pass 2: scatter.
__global__ void __launch_bounds__(kThreads) k_boundary_scatter(const gbf_model m, gbf_arrays a, const double* scratch) {
  const GbfGeo g = gbf_geo(m);
  const size_t nb = gbf_boundary_count(g);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nb; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    gbf_boundary_cell(g, t, i, j, k);
    size_t c = gbf_idx(g, i, j, k);
    a.S2[c] = scratch[t];
    a.P1[c] = scratch[nb + t];
  }
}

// Scratch of gbf_boundary_f64_noalloc: a fixed array of this library in
// device memory, 8 MiB, held by every GPU that loads the library until the
// process exits. In host code the name is only a stand-in for the array, not
// its device address: host code passes the address that
// cudaGetSymbolAddress returns for the current device (noalloc_scratch).
constexpr size_t kNoAllocScratchDoubles = (size_t)1 << 20;
static __device__ __align__(256) double g_noalloc_scratch[kNoAllocScratchDoubles];

constexpr int kNoAllocMaxDevices = 64;
std::mutex g_noalloc_mu;
// Per device: the array's address and the id of the CUDA context it was looked
// up in. A context that is destroyed (cudaDeviceReset, a reset of the primary
// context) and created again may load the library's module elsewhere, so the
// address is valid only while the context it came from is current.
double* g_noalloc_ptr[kNoAllocMaxDevices] = {};
unsigned long long g_noalloc_ctx[kNoAllocMaxDevices] = {};
PFN_cuCtxGetCurrent_v4000 g_ctx_current = nullptr;
PFN_cuCtxGetId_v12000 g_ctx_id = nullptr;
bool g_ctx_queries_resolved = false;

// Id of the calling thread's current CUDA context (cuCtxGetId: unique for the
// life of the process), or 0 when no context is current or the driver cannot
// tell. The driver functions are reached through the runtime's entry-point
// query, so libgbflow does not link libcuda. Called with g_noalloc_mu held.
unsigned long long current_context_id() {
  if (!g_ctx_queries_resolved) {
    g_ctx_queries_resolved = true;
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 4000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_current = (PFN_cuCtxGetCurrent_v4000)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_ctx_id = (PFN_cuCtxGetId_v12000)f;
  }
  if (!g_ctx_current || !g_ctx_id) return 0;
  CUcontext c = nullptr;
  if (g_ctx_current(&c) != CUDA_SUCCESS || !c) return 0;
  unsigned long long id = 0;
  return g_ctx_id(c, &id) == CUDA_SUCCESS ? id : 0;
}

// Device address of g_noalloc_scratch on the current device, looked up with
// that device current (cudaGetSymbolAddress) on the first call, and again
// whenever the current context is not the one the address came from (or
// cannot be identified); otherwise the cached address.
int noalloc_scratch(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return gbf_cuda_check(e, "gbf_boundary_f64_noalloc: cudaGetDevice");
  if (dev < 0 || dev >= kNoAllocMaxDevices) return gbf_fail(GBF_ERR_ARG, "gbf_boundary_f64_noalloc: device index");
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  const unsigned long long ctx = current_context_id();
  if (!g_noalloc_ptr[dev] || ctx == 0 || ctx != g_noalloc_ctx[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) return gbf_cuda_check(e != cudaSuccess ? e : cudaErrorInvalidSymbol,
                                                      "gbf_boundary_f64_noalloc: cudaGetSymbolAddress");
    g_noalloc_ptr[dev] = (double*)p;
    g_noalloc_ctx[dev] = current_context_id();  // the lookup made a context current if none was
  }
  *out = g_noalloc_ptr[dev];
  return GBF_OK;
}

int check_model(const gbf_model* m, const char* where) {
  if (!m || m->nx < 3 || m->ny < 3 || m->nz < 3) return gbf_fail(GBF_ERR_ARG, where);
  return GBF_OK;
}

int launched(const char* where) {
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GBF_OK : gbf_cuda_check(e, where);
}

// Start-of-step phase masses of interior cells from a state (P, S): what
// assign_rS_nr leaves in roS1_old, roS2_old (cpu.cpp:222-225, 286-287) with
// the densities of assign_ro1_ro2 at P2 = P1 (cpu.cpp:63-74). FP64 state, or
// the split state (dP from the hydrostatic profile, S in FP32) when P is NULL.
// Boundary cells get 0.
__global__ void __launch_bounds__(kThreads) k_roS_old(const gbf_model m, const double* P, const double* S,
                                                      const float* dPf, const float* Sf, double* o1, double* o2) {
  const GbfGeo g = gbf_geo(m);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.n; c += (size_t)gridDim.x * blockDim.x) {
    const int i = (int)(c % g.nx), j = (int)((c / g.nx) % g.ny), k = (int)(c / g.pl);
    if (gbf_is_boundary(g, i, j, k)) {
      o1[c] = 0.;
      o2[c] = 0.;
      continue;
    }
    const double p = P ? P[c] : gbf_p_hydrostatic(m, j) + (double)dPf[c];
    const double s = S ? S[c] : (double)Sf[c];
    const double ro1 = m.ro01 * (1. + (m.beta1) * (p - m.P_atm));
    const double ro2 = m.ro02 * (1. + (m.beta2) * (p - m.P_atm));
    o1[c] = ro1 * (1 - s);
    o2[c] = ro2 * s;
  }
}

}  // namespace

int gbf_roS_old_launch(const gbf_model& m, const double* P, const double* S, const float* dPf, const float* Sf,
                       double* o1, double* o2, cudaStream_t st) {
  k_roS_old<<<gbf_grid_for(gbf_geo(m).n, kThreads), kThreads, 0, st>>>(m, P, S, dPf, Sf, o1, o2);
  GBF_CUDA(cudaGetLastError());
  return GBF_OK;
}

extern "C" {

int gbf_props_f64(const gbf_model* m, gbf_arrays a, gbf_cells cells, void* stream) {
  if (int s = check_model(m, "gbf_props_f64")) return s;
  k_props<<<gbf_grid_for(gbf_geo(*m).n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(*m, a, cells);
  return launched("gbf_props_f64");
}

int gbf_velocity_f64(const gbf_model* m, gbf_arrays a, void* stream) {
  if (int s = check_model(m, "gbf_velocity_f64")) return s;
  k_velocity<<<gbf_grid_for(gbf_geo(*m).n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(*m, a);
  return launched("gbf_velocity_f64");
}

int gbf_mass_f64(const gbf_model* m, gbf_arrays a, gbf_cells cells, void* stream) {
  if (int s = check_model(m, "gbf_mass_f64")) return s;
  size_t nint = (size_t)(m->nx - 2) * (m->ny - 2) * (m->nz - 2);
  k_mass<<<gbf_grid_for(nint, kThreads), kThreads, 0, (cudaStream_t)stream>>>(*m, a, cells);
  return launched("gbf_mass_f64");
}

int gbf_newton_f64(const gbf_model* m, gbf_arrays a, gbf_cells cells, void* stream) {
  if (int s = check_model(m, "gbf_newton_f64")) return s;
  size_t nint = (size_t)(m->nx - 2) * (m->ny - 2) * (m->nz - 2);
  k_newton<<<gbf_grid_for(nint, kThreads), kThreads, 0, (cudaStream_t)stream>>>(*m, a, cells);
  return launched("gbf_newton_f64");
}

size_t gbf_boundary_scratch_doubles(const gbf_model* m) {
  if (!m || m->nx < 3 || m->ny < 3 || m->nz < 3) return 0;
  return 2 * gbf_boundary_count(gbf_geo(*m));
}

int gbf_boundary_f64(const gbf_model* m, gbf_arrays a, double* scratch, void* stream) {
  if (int s = check_model(m, "gbf_boundary_f64")) return s;
  if (!scratch) return gbf_fail(GBF_ERR_ARG, "gbf_boundary_f64: scratch");
  size_t nb = gbf_boundary_count(gbf_geo(*m));
  unsigned grid = gbf_grid_for(nb, kThreads);
  k_boundary_gather<<<grid, kThreads, 0, (cudaStream_t)stream>>>(*m, a, scratch);
  k_boundary_scatter<<<grid, kThreads, 0, (cudaStream_t)stream>>>(*m, a, scratch);
  return launched("gbf_boundary_f64");
}

// The boundary pass for callers that cannot allocate device memory when they
// apply the boundary conditions. Same kernels and results as
// gbf_boundary_f64; the gather scratch is the library's fixed device array
// g_noalloc_scratch instead of a caller buffer. Allocates nothing: no
// cudaMalloc, cudaFree or allocating library routine. The first call on a
// device looks up the array's address there (cudaGetSymbolAddress), and so
// does the first call after that device's context was destroyed and created
// again, so make those calls before any stream capture. Every call on a device uses the
// same array, which keeps the last call's contents: the gather fills every
// slot the scatter reads, so nothing needs clearing, and calls that overlap
// on the same GPU (from several streams or host threads) race on it.
int gbf_boundary_f64_noalloc(const gbf_model* m, gbf_arrays a, void* stream) {
  if (int s = check_model(m, "gbf_boundary_f64_noalloc")) return s;
  const size_t nb = gbf_boundary_count(gbf_geo(*m));
  if (2 * nb > kNoAllocScratchDoubles)
    return gbf_fail(GBF_ERR_ARG, "gbf_boundary_f64_noalloc: more than 524288 boundary cells (its fixed 8 MiB "
                                 "scratch holds 2 doubles per boundary cell); use gbf_boundary_f64");
  double* scratch = nullptr;
  if (int s = noalloc_scratch(&scratch)) return s;
  const unsigned grid = gbf_grid_for(nb, kThreads);
  k_boundary_gather<<<grid, kThreads, 0, (cudaStream_t)stream>>>(*m, a, scratch);
  k_boundary_scatter<<<grid, kThreads, 0, (cudaStream_t)stream>>>(*m, a, scratch);
  return launched("gbf_boundary_f64_noalloc");
}

}  // extern "C"
