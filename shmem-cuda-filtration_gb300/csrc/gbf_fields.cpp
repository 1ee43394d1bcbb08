// gbf_fields.cpp — seeded synthetic cell fields (permeability, porosity).
//
// The reference has a 2-entry media table only (defines.h:22-26); the
// heterogeneous workloads need per-cell fields, generated here on the host
// deterministically from a seed, independent of the thread count:
//   * SplitMix64 (Steele, Lea, Flood 2014) as the random stream, one stream
//     per cell index (counter-based: value = mix(seed, cell)), so any slice
//     of the grid can be generated by any thread;
//   * Box-Muller transform for standard normals;
//   * separable Gaussian smoothing (sigma = correlation length in cells,
//     truncated at 3 sigma, mirrored at the faces), then renormalisation of
//     the smoothed field to zero mean and unit variance;
//   * ln K = ln(K_geo) + sigma_lnK * z, K = exp(ln K) rounded to FP32.
// It also holds the stability bound gbf_stable_dt, which the workloads derive
// their time step from.
//
// The file needs the host compiler only. Built with GBF_INPUTS_STANDALONE it
// makes a small library of its own (libgbf_inputs.so, oracle/Makefile), so
// that a CPU-only caller — the timed reference CPU run — generates the same
// inputs without loading libgbflow; both builds use -ffp-contract=off and give
// the same bits (tested).
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <thread>
#include <vector>

#ifdef GBF_INPUTS_STANDALONE
#include "gbflow.h"
// Alone, errors are returned without libgbflow's sticky status.
static int gbf_fail(int s, const char*) { return s; }
#else
#include "gbf_internal.h"
#endif

namespace {

inline uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
// Uniform in (0, 1): 53 random bits, never 0.
inline double u01(uint64_t seed, uint64_t ctr) {
  uint64_t r = splitmix64(seed * 0x9E3779B97F4A7C15ull ^ splitmix64(ctr));
  return ((double)(r >> 11) + 0.5) * (1.0 / 9007199254740992.0);
}
inline double normal(uint64_t seed, uint64_t cell) {
  double u1 = u01(seed, 2 * cell), u2 = u01(seed, 2 * cell + 1);
  return sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
}

template <class F>
void parallel_for(size_t n, F f) {
  unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
  if (n < 4096) nt = 1;
  std::vector<std::thread> th;
  size_t chunk = (n + nt - 1) / nt;
  for (unsigned t = 0; t < nt; t++) {
    size_t a = t * chunk, b = std::min(n, a + chunk);
    if (a >= b) break;
    th.emplace_back([=] { for (size_t q = a; q < b; q++) f(q); });
  }
  for (auto& x : th) x.join();
}

inline int mirror(int i, int n) {
  while (i < 0 || i >= n) {
    if (i < 0) i = -i - 1;
    if (i >= n) i = 2 * n - i - 1;
  }
  return i;
}

// One separable pass along axis `ax` (0 = i, 1 = j, 2 = k) of a (nx, ny, nz) field.
void smooth_axis(const std::vector<double>& in, std::vector<double>& out, int nx, int ny, int nz, int ax,
                 const std::vector<double>& w, int r) {
  const int dims[3] = {nx, ny, nz};
  const size_t strides[3] = {1, (size_t)nx, (size_t)nx * ny};
  const int n = dims[ax];
  const size_t st = strides[ax];
  const size_t lines = (size_t)nx * ny * nz / n;
  parallel_for(lines, [&](size_t L) {
    // base index of line L: enumerate the two other axes
    size_t base;
    if (ax == 0) base = L * nx;
    else if (ax == 1) base = (L % nx) + (L / nx) * (size_t)nx * ny;
    else base = L;
    for (int p = 0; p < n; p++) {
      double acc = 0;
      for (int q = -r; q <= r; q++) acc += w[q + r] * in[base + (size_t)mirror(p + q, n) * st];
      out[base + (size_t)p * st] = acc;
    }
  });
}

}  // namespace

extern "C" {

// Log-normal permeability: geometric mean K_geo, log-standard deviation
// sigma_lnK, Gaussian correlation length corr_cells (0: white noise).
int gbf_fill_lognormal_K(int nx, int ny, int nz, uint64_t seed, double K_geo, double sigma_lnK, double corr_cells,
                         float* K_out) {
  if (nx < 1 || ny < 1 || nz < 1 || !K_out || !(K_geo > 0) || !(sigma_lnK >= 0) || !(corr_cells >= 0))
    return gbf_fail(GBF_ERR_ARG, "gbf_fill_lognormal_K");
  const size_t n = (size_t)nx * ny * nz;
  std::vector<double> a(n), b(n);
  parallel_for(n, [&](size_t c) { a[c] = normal(seed, c); });
  if (corr_cells > 0) {
    int r = (int)ceil(3.0 * corr_cells);
    std::vector<double> w(2 * r + 1);
    double ws = 0;
    for (int q = -r; q <= r; q++) ws += (w[q + r] = exp(-0.5 * (q / corr_cells) * (q / corr_cells)));
    for (auto& x : w) x /= ws;
    smooth_axis(a, b, nx, ny, nz, 0, w, r);
    smooth_axis(b, a, nx, ny, nz, 1, w, r);
    smooth_axis(a, b, nx, ny, nz, 2, w, r);
    a.swap(b);
  }
  double mean = 0, var = 0;
  for (size_t c = 0; c < n; c++) mean += a[c];
  mean /= (double)n;
  for (size_t c = 0; c < n; c++) var += (a[c] - mean) * (a[c] - mean);
  double sd = n > 1 ? sqrt(var / (double)(n - 1)) : 1.0;
  if (!(sd > 0)) sd = 1.0;
  const double lk = log(K_geo);
  parallel_for(n, [&](size_t c) { K_out[c] = (float)exp(lk + sigma_lnK * (a[c] - mean) / sd); });
  return GBF_OK;
}

// Porosity phi = base + amp * U(-1, 1) per cell.
int gbf_fill_porosity(int nx, int ny, int nz, uint64_t seed, double base, double amp, float* phi_out) {
  if (nx < 1 || ny < 1 || nz < 1 || !phi_out || !(base - fabs(amp) > 0) || !(base + fabs(amp) <= 1))
    return gbf_fail(GBF_ERR_ARG, "gbf_fill_porosity");
  const size_t n = (size_t)nx * ny * nz;
  const uint64_t s = splitmix64(seed ^ 0x5bd1e995ull);
  parallel_for(n, [&](size_t c) { phi_out[c] = (float)(base + amp * (2.0 * u01(s, c) - 1.0)); });
  return GBF_OK;
}

// Explicit-scheme bound of the pressure equation. Its diffusivity is
// D = K lambda_t(S) / (phi c_t(S)) with the total mobility
// lambda_t = kr1/mu1 + kr2/mu2 (Brooks-Corey, as in cpu.cpp:60-62) and the
// total compressibility c_t = (1 - S) beta1 + S beta2, maximised over the
// saturations the source can produce (S in [0, S2_gr] for the reference's
// Dirichlet patch, [0, 1 - S_wr) for a mass rate); then
// dt <= 1 / (2 D (1/h1^2 + kv/h2^2 + 1/h3^2)). It bounds the pressure
// diffusion only (advection limits are far looser in the configurations used
// here).
double gbf_stable_dt(const gbf_model* m, const gbf_cells* cells, double safety) {
  if (!m) return 0;
  const size_t n = (size_t)m->nx * m->ny * m->nz;
  double ratio[2] = {0, 0};  // max over S of lambda_t / c_t, per media
  for (int md = 0; md < 2; md++) {
    const double swr = m->S_wr[md], lam = m->lambda[md];
    const double scap = (m->source_mode == GBF_SOURCE_DIRICHLET_PATCH) ? fmin(m->S2_gr, 1 - swr) : 1 - swr;
    for (int q = 0; q <= 256; q++) {
      const double s = scap * q / 256.0;
      const double se = fmax(0.0, (1 - s - swr) / (1 - swr));
      const double kr1 = pow(se, (2 + 3 * lam) / lam);
      const double kr2 = (1 - se) * (1 - se) * (1 - pow(se, (2 + lam) / lam));
      const double ct = (1 - s) * m->beta1 + s * m->beta2;
      if (ct > 0) ratio[md] = fmax(ratio[md], (kr1 / m->mu1 + kr2 / m->mu2) / ct);
    }
  }
  double dmax = 0;
  const bool per_cell = cells && (cells->K || cells->phi);
  if (!per_cell) {
    for (int md = 0; md < 2; md++) {
      bool used = !(cells && cells->media) ? (md == 0) : false;
      if (cells && cells->media)
        for (size_t c = 0; c < n && !used; c++) used = cells->media[c] == md;
      if (used) dmax = fmax(dmax, m->K[md] * ratio[md] / m->m[md]);
    }
  } else {
    for (size_t c = 0; c < n; c++) {
      int md = (cells->media) ? cells->media[c] : 0;
      double K = cells->K ? (double)cells->K[c] : m->K[md];
      double phi = cells->phi ? (double)cells->phi[c] : m->m[md];
      dmax = fmax(dmax, K * ratio[md] / phi);
    }
  }
  double inv = 1.0 / (m->h1 * m->h1) + m->kv / (m->h2 * m->h2) + 1.0 / (m->h3 * m->h3);
  if (dmax <= 0 || inv <= 0) return 0;
  return safety / (2.0 * dmax * inv);
}

}  // extern "C"
