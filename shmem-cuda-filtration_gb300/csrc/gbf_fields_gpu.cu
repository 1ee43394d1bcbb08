// gbf_fields_gpu.cu — the seeded synthetic cell fields of gbf_fields.cpp
// generated on the device, from the same counter-based SplitMix64 streams
// (value = mix(seed, cell index)), Box-Muller normals, separable Gaussian
// smoothing (truncated at 3 sigma, mirrored at the faces), renormalisation
// and K = exp(ln K_geo + sigma_lnK z) in FP32. Porosity is bit-identical to
// the host generator (integer mixing, one rounded multiply-add chain
// without contraction). The permeability differs from the host field only
// where the host libm and CUDA's log/cos/exp round the last bit differently
// and that moves the FP32 rounding of K: at most 1 FP32 ulp in a few cells.
#include <stdint.h>

#include <vector>

#include "gbf_internal.h"

namespace {

constexpr int kThreads = 256;
constexpr int kMaxTaps = 1024;
__constant__ double c_w[kMaxTaps];

__device__ __forceinline__ uint64_t splitmix64(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}
__device__ __forceinline__ double u01(uint64_t seed, uint64_t ctr) {
  const uint64_t r = splitmix64(seed * 0x9E3779B97F4A7C15ull ^ splitmix64(ctr));
  return __dmul_rn(__dadd_rn((double)(r >> 11), 0.5), 1.0 / 9007199254740992.0);
}
__device__ __forceinline__ int mirror(int i, int n) {
  while (i < 0 || i >= n) {
    if (i < 0) i = -i - 1;
    if (i >= n) i = 2 * n - i - 1;
  }
  return i;
}

__global__ void k_normals(size_t n, uint64_t seed, double* a) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const double u1 = u01(seed, 2 * c), u2 = u01(seed, 2 * c + 1);
    a[c] = sqrt(-2.0 * log(u1)) * cos(6.283185307179586 * u2);
  }
}

// One separable pass along axis `ax` (stride `st`, length `len`); taps in c_w.
__global__ void k_smooth(const double* in, double* out, int nx, int ny, int nz, int ax, int r) {
  const size_t n = (size_t)nx * ny * nz;
  const int len = ax == 0 ? nx : ax == 1 ? ny : nz;
  const size_t st = ax == 0 ? 1 : ax == 1 ? (size_t)nx : (size_t)nx * ny;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const int p = (int)((c / st) % (size_t)len);
    const size_t base = c - (size_t)p * st;
    double acc = 0;
    for (int q = -r; q <= r; q++) acc += c_w[q + r] * in[base + (size_t)mirror(p + q, len) * st];
    out[c] = acc;
  }
}

// Fixed-shape two-level sums (deterministic for a size): per-block partials of
// x (mode 0) or (x - mean)^2 (mode 1), then one block over the partials.
__global__ void k_partial(const double* a, size_t n, const double* mean, int mode, double* part) {
  __shared__ double red[kThreads];
  double s = 0;
  const double mu = mode ? *mean : 0.0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const double v = a[c] - mu;
    s += mode ? v * v : a[c];
  }
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}
__global__ void k_finish(const double* part, int nb, double div, double* out) {
  __shared__ double red[kThreads];
  double s = 0;
  for (int q = threadIdx.x; q < nb; q += kThreads) s += part[q];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0] / div;
}

__global__ void k_lognormal(const double* a, size_t n, const double* stats, double lk, double sigma, float* K) {
  const double mean = stats[0];
  double sd = stats[1] > 0 ? sqrt(stats[1]) : 1.0;
  if (n <= 1) sd = 1.0;
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x)
    K[c] = (float)exp(lk + sigma * (a[c] - mean) / sd);
}

__global__ void k_porosity(size_t n, uint64_t s, double base, double amp, float* phi) {
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
    const double u = __dsub_rn(__dmul_rn(2.0, u01(s, c)), 1.0);
    phi[c] = (float)__dadd_rn(base, __dmul_rn(amp, u));
  }
}

}  // namespace

extern "C" {

int gbf_fill_lognormal_K_device(int nx, int ny, int nz, uint64_t seed, double K_geo, double sigma_lnK,
                                double corr_cells, float* d_K, void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || !d_K || !(K_geo > 0) || !(sigma_lnK >= 0) || !(corr_cells >= 0))
    return gbf_fail(GBF_ERR_ARG, "gbf_fill_lognormal_K_device");
  const int r = corr_cells > 0 ? (int)ceil(3.0 * corr_cells) : 0;
  if (2 * r + 1 > kMaxTaps) return gbf_fail(GBF_ERR_ARG, "gbf_fill_lognormal_K_device: correlation length");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t n = (size_t)nx * ny * nz;
  const unsigned grid = gbf_grid_for(n, kThreads);
  double *a = nullptr, *b = nullptr, *part = nullptr;
  GBF_CUDA(cudaMallocAsync((void**)&a, n * sizeof(double), st));
  GBF_CUDA(cudaMallocAsync((void**)&b, n * sizeof(double), st));
  GBF_CUDA(cudaMallocAsync((void**)&part, (grid + 2) * sizeof(double), st));
  double* stats = part + grid;  // mean, variance
  k_normals<<<grid, kThreads, 0, st>>>(n, seed, a);
  if (r > 0) {
    std::vector<double> w(2 * r + 1);
    double ws = 0;
    for (int q = -r; q <= r; q++) ws += (w[q + r] = exp(-0.5 * (q / corr_cells) * (q / corr_cells)));
    for (auto& x : w) x /= ws;
    GBF_CUDA(cudaMemcpyToSymbolAsync(c_w, w.data(), w.size() * sizeof(double), 0, cudaMemcpyHostToDevice, st));
    k_smooth<<<grid, kThreads, 0, st>>>(a, b, nx, ny, nz, 0, r);
    k_smooth<<<grid, kThreads, 0, st>>>(b, a, nx, ny, nz, 1, r);
    k_smooth<<<grid, kThreads, 0, st>>>(a, b, nx, ny, nz, 2, r);
    std::swap(a, b);
  }
  k_partial<<<grid, kThreads, 0, st>>>(a, n, nullptr, 0, part);
  k_finish<<<1, kThreads, 0, st>>>(part, (int)grid, (double)n, stats);
  k_partial<<<grid, kThreads, 0, st>>>(a, n, stats, 1, part);
  k_finish<<<1, kThreads, 0, st>>>(part, (int)grid, n > 1 ? (double)(n - 1) : 1.0, stats + 1);
  k_lognormal<<<grid, kThreads, 0, st>>>(a, n, stats, log(K_geo), sigma_lnK, d_K);
  GBF_CUDA(cudaGetLastError());
  cudaFreeAsync(a, st);
  cudaFreeAsync(b, st);
  cudaFreeAsync(part, st);
  GBF_CUDA(cudaStreamSynchronize(st));  // the weights' host buffer dies here
  return GBF_OK;
}

int gbf_fill_porosity_device(int nx, int ny, int nz, uint64_t seed, double base, double amp, float* d_phi,
                             void* stream) {
  if (nx < 1 || ny < 1 || nz < 1 || !d_phi || !(base - fabs(amp) > 0) || !(base + fabs(amp) <= 1))
    return gbf_fail(GBF_ERR_ARG, "gbf_fill_porosity_device");
  const size_t n = (size_t)nx * ny * nz;
  // the host generator's stream seed: splitmix64(seed ^ 0x5bd1e995)
  uint64_t x = (seed ^ 0x5bd1e995ull) + 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  const uint64_t s = x ^ (x >> 31);
  k_porosity<<<gbf_grid_for(n, kThreads), kThreads, 0, (cudaStream_t)stream>>>(n, s, base, amp, d_phi);
  GBF_CUDA(cudaGetLastError());
  return GBF_OK;
}

}  // extern "C"
