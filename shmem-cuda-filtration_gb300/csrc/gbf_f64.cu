// gbf_f64.cu — plain FP64 step of one domain, fused into two passes plus a
// face pass (per-cell code in gbf_f64_cell.cuh).
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
#include "gbf_f64_cell.cuh"

namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads) k_f64_props(const gbf_model m, const GbfDerived d, const gbf_cells cells,
                                                        const GbfF64Step s, const int flags) {
  const GbfGeo g = gbf_geo(m);
  for (size_t c = blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < g.n; c += (size_t)gridDim.x * blockDim.x)
    gbf_f64_props_cell(m, d, cells, s, flags, g, c);
}

__global__ void __launch_bounds__(kThreads) k_f64_flux_newton(const gbf_model m, const GbfDerived d,
                                                              const gbf_cells cells, const GbfF64Step s) {
  const GbfGeo g = gbf_geo(m);
  const size_t ix = (size_t)g.nx - 2, iy = (size_t)g.ny - 2;
  const size_t nint = ix * iy * (size_t)(g.nz - 2);
  double msum1 = 0., msum2 = 0.;
  unsigned bad = 0;
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nint; t += (size_t)gridDim.x * blockDim.x) {
    const int i = 1 + (int)(t % ix), j = 1 + (int)((t / ix) % iy), k = 1 + (int)(t / (ix * iy));
    gbf_f64_flux_newton_cell(m, d, cells, s, g, i, j, k, msum1, msum2, bad);
  }
  if (bad) atomicOr(s.status, GBF_DEV_NONFINITE);
  if (s.mass_partials) gbf_block_sum2<kThreads>(msum1, msum2, d.V, s.mass_partials + 2 * blockIdx.x);
}

__global__ void __launch_bounds__(kThreads) k_f64_boundary(const gbf_model m, const GbfF64Step s) {
  const GbfGeo g = gbf_geo(m);
  const size_t nb = gbf_boundary_count(g);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nb; t += (size_t)gridDim.x * blockDim.x)
    gbf_f64_boundary_cell(m, s, g, t);
}

}  // namespace

// Sum per-block partial pairs [2q, 2q+1] in a fixed order (one block of 256).
__global__ void gbf_k_mass_tail(const double* partials, int nblocks, double* out) {
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
    gbf_k_mass_tail<<<1, 256, 0, st>>>(s.mass_partials, (int)fg, mass_out);
    gbf_timer_end(tm, GBF_K_MASS_TAIL, e, st);
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? GBF_OK : gbf_cuda_check(err, "gbf_f64_launch_step");
}
