// gbf_split.cu — split-precision step: FP32 pressure, saturation, K, phi and
// fluxes; FP64 (or FP32-pair) per-cell phase masses and one wide-precision
// residual per cell.
//
// State (per cell):
//   dP  = P - P_hs(j), FP32, with P_hs(j) = P_atm + j rho01 g h2 the
//         hydrostatic profile of the initial state (main.cpp:114). Vertical
//         potentials then read -(dP(j+1) - dP(j))/h2 + (rho_c - rho01) g: the
//         two large hydrostatic terms cancel exactly before anything is rounded.
//   S   = S2, FP32.
//   M1, M2 (interior cells): the phase masses per pore volume the
//         reference's mass update starts from, ro1 (1 - S2) and ro2 S2 with
//         ro2 at P2 = P1 (cpu.cpp:224-225), in FP64 (GBF_PREC_SPLIT), as an
//         unevaluated sum of two FP32 (GBF_PREC_SPLIT_DF), or as FP32 defects
//         over c1(j) (1 - S), c2(j) S (GBF_PREC_SPLIT_DEFECT).
// The tile routine (gbf_split_tile.cuh) does the fused update of one column
// tile; this file holds the single-domain kernels and the host side.
#include <math.h>

#include <algorithm>

#include "gbf_split_tile.cuh"

GbfPatchConsts gbf_patch_consts(const gbf_model& m) {
  GbfPatchConsts P = {};
  if (m.source_mode != GBF_SOURCE_DIRICHLET_PATCH || m.source < 0) return P;
  P.n = 2 * m.source + 1;
  P.i0 = m.nx / 2 - m.source;
  P.k0 = m.nz / 2 - m.source;
  P.S2 = m.S2_gr;
  P.nmr2 = -m.ro02 / m.mu2;
  P.gh2 = m.g * m.h2;
  P.wy = m.dt * m.kv / (m.h2 * m.h2);
  for (int md = 0; md < 2; md++) {
    P.K[md] = m.K[md];
    P.se_b[md] = -1.0 / (1.0 - m.S_wr[md]);
    P.e2[md] = (2. + m.lambda[md]) / m.lambda[md];
  }
  return P;
}

GbfSplitConsts gbf_split_consts(const gbf_model& m) {
  GbfSplitConsts C = {};
  C.nx = m.nx; C.ny = m.ny; C.nz = m.nz;
  C.noflow_bottom = (m.bc_mode == GBF_BC_HYDROSTATIC_SIDES);
  const double V = m.h1 * m.h2 * m.h3;
  double src = 0.0;
  if (m.source_mode == GBF_SOURCE_RATE && m.rate_cells > 0) {
    C.rn = m.rate_cells;
    C.ri0 = m.nx / 2 - m.rate_cells / 2;
    C.rk0 = m.nz / 2 - m.rate_cells / 2;
    src = m.rate / (double)(m.rate_cells * m.rate_cells) / V;
  } else {  // the cells under the Dirichlet patch (the PATCH tiles; gbf_patch_consts)
    const GbfPatchConsts P = gbf_patch_consts(m);
    C.rn = P.n;
    C.ri0 = P.i0;
    C.rk0 = P.k0;
  }
  const double H = m.ro01 * m.g * m.h2;
  C.H = (float)H;
  C.ro01 = (float)m.ro01; C.ro02 = (float)m.ro02; C.beta1 = (float)m.beta1; C.beta2 = (float)m.beta2;
  C.bmax = C.beta1 > C.beta2 ? C.beta1 : C.beta2;
  C.cfl1 = (float)(1.0 / m.ro01); C.cfl2 = (float)(1.0 / m.ro02);
  C.nmr1 = (float)(-m.ro01 / m.mu1);
  C.nmr2 = (float)(-m.ro02 / m.mu2);
  C.ro01b1 = (float)(m.ro01 * m.beta1);
  C.ro02b2 = (float)(m.ro02 * m.beta2);
  for (int md = 0; md < 2; md++) {
    const double lam = m.lambda[md], swr = m.S_wr[md];
    C.K[md] = (float)m.K[md];
    C.m[md] = (float)m.m[md];
    C.se_b[md] = (float)(-1.0 / (1.0 - swr));
    C.e1[md] = (float)((2. + 3. * lam) / lam);
    C.e2[md] = (float)((2. + lam) / lam);
    C.m_inv_lam[md] = (float)(-1. / lam);
    C.inv_lam_1mswr[md] = (float)(1.0 / (lam * (1.0 - swr)));
    C.P_d[md] = (float)m.P_d[md];
  }
  C.H_d = H; C.beta1_d = m.beta1; C.beta2_d = m.beta2; C.ro01_d = m.ro01; C.ro02_d = m.ro02;
  C.dtsrc_d = m.dt * src;
  C.V = V;
  C.ro01b1_d = m.ro01 * m.beta1;
  C.ro02b2_d = m.ro02 * m.beta2;
  C.ro01b1_lo = (float)(C.ro01b1_d - (double)C.ro01b1);
  C.ro02b2_lo = (float)(C.ro02b2_d - (double)C.ro02b2);
  C.gh1 = (float)(m.g * m.ro01 * m.beta1 * m.h2);
  C.gh2 = (float)(m.g * m.ro02 * m.beta2 * m.h2);
  C.ghd = (float)(m.g * (m.ro02 - m.ro01) * m.h2);
  C.wx = (float)(m.dt / (m.h1 * m.h1));
  C.wy = (float)(m.dt * m.kv / (m.h2 * m.h2));
  C.wz = (float)(m.dt / (m.h3 * m.h3));
  C.H_df = gbf_df_from_double(H);
  C.beta1_df = gbf_df_from_double(m.beta1);
  C.beta2_df = gbf_df_from_double(m.beta2);
  C.ro01_df = gbf_df_from_double(m.ro01);
  C.ro02_df = gbf_df_from_double(m.ro02);
  C.dtsrc_df = gbf_df_from_double(C.dtsrc_d);
  for (int md = 0; md < 2; md++) {
    C.m_d[md] = m.m[md];
    C.m_df[md] = gbf_df_from_double(m.m[md]);
    C.dtsrc_m_d[md] = C.dtsrc_d / m.m[md];
    C.dtsrc_m_df[md] = gbf_df_from_double(C.dtsrc_m_d[md]);
  }
  return C;
}

namespace {

constexpr int kThreads = 256;

int tiles_x(const GbfSplitConsts& C) { return (C.nx - 2 + kSplitTX - 1) / kSplitTX; }
int tiles_y(const GbfSplitConsts& C) { return (C.ny - 2 + kSplitTY - 1) / kSplitTY; }
// x-pair tiles (TMA staging): 64 x 8 cells from x0 = 64 t, t such that x0 <= nx - 2
constexpr int kPairTX = 64, kPairTY = 8;
__host__ __device__ int tiles_x2(const GbfSplitConsts& C) { return (C.nx - 1 + kPairTX - 1) / kPairTX; }
__host__ __device__ int tiles_y2(const GbfSplitConsts& C) { return (C.ny - 2 + kPairTY - 1) / kPairTY; }

// The plain-load tile on one grid (grids without TMA staging). Block b runs
// tile b mod (tiles of a chunk layer) of the k chunk kc0 + b / (tiles of a
// layer), kchunk planes from 1 + kchunk kc; G.mass_partials is that launch's
// first partial.
template <int MR, bool CFL, bool PATCH>
__global__ void __launch_bounds__(kSplitThreads, 4) k_split_step(const GbfSplitConsts C, const GbfSplitGrid G,
                                                              const int kchunk, const int kc0) {
  __shared__ GbfSplitPlane pl[2];
  const int ntx = (C.nx - 2 + kSplitTX - 1) / kSplitTX, nty = (C.ny - 2 + kSplitTY - 1) / kSplitTY;
  const int b = blockIdx.x;
  const int tx = b % ntx, ty = (b / ntx) % nty, kc = kc0 + b / (ntx * nty);
  const int k0 = 1 + kc * kchunk;
  const int k1 = min(k0 + kchunk, C.nz - 1);
  GbfSplitAcc<MR> acc;
  split_tile<MR, kSplitTX, kSplitTY, false, CFL, PATCH>(C, G, 1 + tx * kSplitTX, 1 + ty * kSplitTY, k0, k1, pl, acc);
  if (acc.bad) atomicOr(G.status, GBF_DEV_NONFINITE);
  if (G.mass_partials) split_block_mass<MR>(acc, C.V, G.mass_partials + 2 * blockIdx.x);
  if constexpr (CFL) split_block_cfl<kSplitThreads>(acc.cfl1, acc.cfl2, G.cfl_out);
}

// The x-pair tile on one grid: one tile (64 x 8 cells, a k range) per CTA,
// blocks mapped to tiles and k chunks as in k_split_step.
template <int MR, bool CFL, bool PATCH>
__global__ void __launch_bounds__(kPairTX / 2 * kPairTY, gbf_pair_ctas(MR)) k_split_step_x2(const GbfSplitConsts C,
                                                                         const GbfSplitGrid G, const int kchunk,
                                                                         const int kc0, const GbfTmaSet* maps,
                                                                         int buf) {
  extern __shared__ __align__(128) unsigned char dyn[];
  using Cta = GbfPairCta<kPairTX, kPairTY, MR>;
  Cta& cta = *reinterpret_cast<Cta*>(dyn);
  if (gbf_smem_u32(dyn) & 127u) {  // the TMA destinations need it; never expected to fire
    if (threadIdx.x == 0) atomicOr(G.status, GBF_DEV_TIMEOUT);
    return;
  }
  const int ntx = tiles_x2(C), nty = tiles_y2(C);
  const int b = blockIdx.x;
  const int tx = b % ntx, ty = (b / ntx) % nty, kc = kc0 + b / (ntx * nty);
  const int k0 = 1 + kc * kchunk;
  const int k1 = min(k0 + kchunk, C.nz - 1);
  if (threadIdx.x == 0) gbf_pair_bars_init(cta.bars);
  __syncthreads();
  unsigned phases = 0;
  GbfSplitAcc<MR> acc;
  split_tile_x2<MR, kPairTX, kPairTY, CFL, kPairTX / 2 * kPairTY, PATCH>(C, G, kPairTX * tx, 1 + kPairTY * ty, k0,
                                                                         k1, cta.bars, cta.body, acc, maps, buf,
                                                                         &phases);
  if (acc.bad) atomicOr(G.status, GBF_DEV_NONFINITE);
  if (G.mass_partials) split_block_mass<MR, kPairTX / 2 * kPairTY>(acc, C.V, G.mass_partials + 2 * blockIdx.x);
  if constexpr (CFL) split_block_cfl<kPairTX / 2 * kPairTY>(acc.cfl1, acc.cfl2, G.cfl_out);
}

// Boundary cells [0, nb) of gbf_boundary_cell's enumeration (all, or all but
// the x faces that the x-pair tile writes).
__global__ void __launch_bounds__(kThreads) k_split_boundary(const gbf_model m, const GbfSplitGrid G, float H,
                                                             size_t nb, int k_lo, int k_hi) {
  const GbfGeo g = gbf_geo(m);
  for (size_t t = blockIdx.x * (size_t)blockDim.x + threadIdx.x; t < nb; t += (size_t)gridDim.x * blockDim.x) {
    int i, j, k;
    gbf_boundary_cell(g, t, i, j, k);
    if (k < k_lo || k >= k_hi) continue;  // planes [k_lo, k_hi) only (a slab of the host pipeline)
    const size_t c = gbf_idx(g, i, j, k);
    G.Sn[c] = gbf_sweep_S<float>(m, g, G.Sn, G.S, i, j, k);
    G.dPn[c] = gbf_split_sweep_dP(m, g, G.dPn, G.dP, i, j, k, H);
  }
}

// Per interior row j: c1(j) times the sum of the row's interior porosities
// (FP64), one block per row.
__global__ void k_defect_k1_rows(const gbf_model m, const float* phi, const int* media, double* rows) {
  __shared__ double red[256];
  const int nx = m.nx, ny = m.ny, nz = m.nz, j = 1 + blockIdx.x;
  const size_t n = (size_t)(nx - 2) * (nz - 2);
  double a = 0.;
  for (size_t t = threadIdx.x; t < n; t += blockDim.x) {
    const int i = 1 + (int)(t % (nx - 2)), k = 1 + (int)(t / (nx - 2));
    const size_t c = (size_t)i + (size_t)j * nx + (size_t)k * nx * ny;
    a += phi ? (double)phi[c] : m.m[media ? media[c] : 0];
  }
  red[threadIdx.x] = a;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) rows[blockIdx.x] = (double)gbf_defect_row(m, j).c1 * red[0];
}
__global__ void k_defect_k1_sum(const double* rows, int nrows, double V, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double a = 0.;
    for (int q = 0; q < nrows; q++) a += rows[q];
    *out = a * V;
  }
}

__global__ void k_split_mass_tail(const double* partials, int nblocks, double* out, double k1v) {
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
  if (threadIdx.x == 0) { out[0] = red[0][0] + k1v; out[1] = red[1][0]; }
}

// rows: the grid's row table (GbfRowConst), or NULL to form each row's
// values per cell (the same values either way).
__global__ void k_split_init(const gbf_model m, const GbfRowConst* rows, const double* P, const double* S,
                             float* dPf, float* Sf, double* M1, double* M2, int mr, size_t c0, size_t c1) {
  const GbfGeo g = gbf_geo(m);
  for (size_t c = c0 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < c1; c += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)((c / g.nx) % g.ny);
    if (rows) gbf_split_init_cell(m, P[c], S[c], rows[j], dPf[c], Sf[c], M1, M2, c, mr);
    else gbf_split_init_cell(m, P[c], S[c], j, dPf[c], Sf[c], M1, M2, c, mr);
  }
}

__global__ void k_split_to_f64(const gbf_model m, const GbfRowConst* rows, const float* dPf, const float* Sf,
                               double* P, double* S, size_t c0, size_t c1) {
  const GbfGeo g = gbf_geo(m);
  for (size_t c = c0 + blockIdx.x * (size_t)blockDim.x + threadIdx.x; c < c1; c += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)((c / g.nx) % g.ny);
    if (P) P[c] = (rows ? rows[j].phs : gbf_p_hydrostatic(m, j)) + (double)dPf[c];
    if (S) S[c] = (double)Sf[c];
  }
}

__global__ void k_split_rows(const gbf_model m, GbfRowConst* rows) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < m.ny; j += gridDim.x * blockDim.x) rows[j] = gbf_row_const(m, j);
}

}  // namespace

// k planes per CTA of a grid of `tiles` column tiles and `nzi` interior
// planes, run with `slots` CTAs resident at a time: the CTAs run in waves,
// and the last wave of an uneven count leaves slots idle. Among k ranges of
// at least 16 planes (or the whole column), take the one with the fewest
// plane-times: waves x (planes per CTA + about 1.5 for the prologue, which
// builds the first plane and loads the plane below it). Grids that fill
// less than one wave may go down to 8 planes per CTA.
int gbf_split_kchunk_waves(long long tiles, int nzi, long long slots) {
  if (nzi < 1) return 1;
  if (slots < 1) slots = 1;
  const int max_chunks = (nzi + 7) / 8;
  int best = nzi;
  double best_cost = 1e300;
  for (int chunks = 1; chunks <= max_chunks; chunks++) {
    const int kc = (nzi + chunks - 1) / chunks;
    const long long ctas = tiles * ((nzi + kc - 1) / kc);
    if (chunks > 1 && kc < 16 && (kc < 8 || ctas > slots)) continue;
    const double cost = (double)((ctas + slots - 1) / slots) * (kc + 1.5);
    if (cost < best_cost - 1e-9) {
      best_cost = cost;
      best = kc;
    }
  }
  return best;
}

// Resident CTAs per SM of the two single-grid tiles (launch bounds and shared memory: the 32x8
// plain-load tile 4, the x-pair tile gbf_pair_ctas: 3 in the defect form, else 2).
int gbf_split_kchunk(const GbfSplitConsts& C) {
  return gbf_split_kchunk_waves((long long)tiles_x(C) * tiles_y(C), C.nz - 2, 4LL * gbf_num_sms());
}
int gbf_split_kchunk_x2(const GbfSplitConsts& C, int mr) {
  return gbf_split_kchunk_waves((long long)tiles_x2(C) * tiles_y2(C), C.nz - 2,
                                (long long)gbf_pair_ctas(mr) * gbf_num_sms());
}

// The step tiles of k chunks [kc0, kc0 + nkc) (kchunk planes each): the
// x-pair tile with TMA staging (maps), else the plain-load tile.
template <int MR, bool CFL, bool PATCH>
int launch_x2(const GbfSplitConsts& C, const GbfSplitGrid& G, const GbfTmaSet* maps, int buf, cudaStream_t st,
              int kchunk, int kc0, int nkc) {
  const unsigned blocks = (unsigned)(tiles_x2(C) * tiles_y2(C) * nkc);
  const int bytes = (int)sizeof(GbfPairCta<kPairTX, kPairTY, MR>);
  GBF_CUDA(cudaFuncSetAttribute(k_split_step_x2<MR, CFL, PATCH>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  k_split_step_x2<MR, CFL, PATCH><<<blocks, kPairTX / 2 * kPairTY, bytes, st>>>(C, G, kchunk, kc0, maps, buf);
  return GBF_OK;
}

namespace {
// The Dirichlet patch's pre-pass, one thread per patch cell (gbf_split_patch_cell).
__global__ void __launch_bounds__(kThreads) k_split_patch(const GbfSplitConsts C, const GbfPatchConsts P,
                                                          const GbfSplitGrid G) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < P.n * P.n; t += gridDim.x * blockDim.x)
    gbf_split_patch_cell(C, P, G, t);
}
}  // namespace

template <int MR, bool PATCH>
int launch_tiles(const GbfSplitConsts& C, const GbfSplitGrid& G, const GbfTmaSet* maps, int buf, cudaStream_t st,
                 int kchunk, int kc0, int nkc) {
  const bool cfl = G.cfl_out != nullptr;
  if (maps)
    return cfl ? launch_x2<MR, true, PATCH>(C, G, maps, buf, st, kchunk, kc0, nkc)
               : launch_x2<MR, false, PATCH>(C, G, maps, buf, st, kchunk, kc0, nkc);
  const unsigned blocks = (unsigned)(tiles_x(C) * tiles_y(C) * nkc);
  if (cfl) k_split_step<MR, true, PATCH><<<blocks, kSplitThreads, 0, st>>>(C, G, kchunk, kc0);
  else k_split_step<MR, false, PATCH><<<blocks, kSplitThreads, 0, st>>>(C, G, kchunk, kc0);
  return GBF_OK;
}

// The tiles under a Dirichlet patch (G.patch_in set) are the PATCH instantiations.
int launch_chunks(const GbfSplitConsts& C, const GbfSplitGrid& G, int mr, const GbfTmaSet* maps, int buf,
                  cudaStream_t st, int kchunk, int kc0, int nkc) {
  auto form = [&](auto tag) {
    constexpr int MR = decltype(tag)::value;
    return G.patch_in ? launch_tiles<MR, true>(C, G, maps, buf, st, kchunk, kc0, nkc)
                      : launch_tiles<MR, false>(C, G, maps, buf, st, kchunk, kc0, nkc);
  };
  return mr == kMassDefect ? form(std::integral_constant<int, kMassDefect>{})
         : mr == kMassDF   ? form(std::integral_constant<int, kMassDF>{})
                           : form(std::integral_constant<int, kMassDefectDF>{});
}
// A step's k chunking: kchunk planes a chunk, and the tiles of a chunk layer.
int step_kchunk(const GbfSplitConsts& C, int mr, const GbfTmaSet* maps) {
  return maps ? gbf_split_kchunk_x2(C, mr) : gbf_split_kchunk(C);
}
long long layer_tiles(const GbfSplitConsts& C, const GbfTmaSet* maps) {
  return maps ? (long long)tiles_x2(C) * tiles_y2(C) : (long long)tiles_x(C) * tiles_y(C);
}

int gbf_split_launch_domain(const gbf_model& m, const GbfSplitConsts& C, const GbfSplitGrid& G, int mr,
                            double* mass_out, cudaStream_t st, GbfTimer* tm, const GbfTmaSet* maps, int buf,
                            double k1v) {
  const int kchunk = step_kchunk(C, mr, maps);
  const int nkc = (C.nz - 2 + kchunk - 1) / kchunk;
  const unsigned blocks = (unsigned)(layer_tiles(C, maps) * nkc);
  cudaEvent_t e = gbf_timer_begin(tm, st);
  if (G.patch_in) {  // the Dirichlet patch's FP64 inflow, timed with the step kernel
    const GbfPatchConsts P = gbf_patch_consts(m);
    k_split_patch<<<gbf_grid_for((size_t)P.n * P.n, kThreads), kThreads, 0, st>>>(C, P, G);
  }
  // TMA staging (maps): the x-pair tile; else the plain-load tile
  if (int s = launch_chunks(C, G, mr, maps, buf, st, kchunk, 0, nkc)) return s;
  gbf_timer_end(tm, GBF_K_SPLIT_STEP, e, st);
  e = gbf_timer_begin(tm, st);
  // one cell per thread (row segments, as the ensembles' face pass walks
  // them, measured 8.6 -> 10.4 us on 256^3: too few warps for a latency-bound pass)
  const size_t nb = maps ? gbf_boundary_count_no_xfaces(gbf_geo(m)) : gbf_boundary_count(gbf_geo(m));
  k_split_boundary<<<gbf_grid_for(nb, kThreads, 4), kThreads, 0, st>>>(m, G, C.H, nb, 0, C.nz);
  gbf_timer_end(tm, GBF_K_SPLIT_BOUNDARY, e, st);
  if (G.mass_partials && mass_out) {
    e = gbf_timer_begin(tm, st);
    k_split_mass_tail<<<1, 256, 0, st>>>(G.mass_partials, (int)blocks, mass_out, gbf_is_defect(mr) ? k1v : 0.0);
    gbf_timer_end(tm, GBF_K_MASS_TAIL, e, st);
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? GBF_OK : gbf_cuda_check(err, "gbf_split_launch_domain");
}

// Mass-partial slots: the larger of the two tilings' CTA counts.
// The host-resident pipeline's slabs (gbf_split_advance_host): one k chunk
// layer of the step each, about 1M cells (16 MB each way) or more, so that a
// slab's copies outlast its few launches, at most 16, at least 4 planes.
constexpr long long kPipeSlabCells = 1ll << 20;
int pipe_slabs(const GbfSplitConsts& C) {
  const long long cells = (long long)C.nx * C.ny * C.nz;
  return (int)std::min(16ll, std::max(1ll, cells / kPipeSlabCells));
}
int pipe_kchunk(const GbfSplitConsts& C) {
  const int s = pipe_slabs(C);
  return std::max(4, (C.nz - 2 + s - 1) / s);
}
bool gbf_split_pipelined(const gbf_model& m) {
  const GbfSplitConsts C = gbf_split_consts(m);
  return pipe_slabs(C) >= 2 && (C.nz - 2 + pipe_kchunk(C) - 1) / pipe_kchunk(C) >= 2;
}

unsigned gbf_split_blocks(const gbf_model& m, int mr) {
  const GbfSplitConsts C = gbf_split_consts(m);
  const int kchunk = gbf_split_kchunk(C), kc2 = gbf_split_kchunk_x2(C, mr), kp = pipe_kchunk(C);
  const unsigned a = (unsigned)(tiles_x(C) * tiles_y(C) * ((C.nz - 2 + kchunk - 1) / kchunk));
  const unsigned b = (unsigned)(tiles_x2(C) * tiles_y2(C) * ((C.nz - 2 + kc2 - 1) / kc2));
  const unsigned p = (unsigned)(std::max(tiles_x(C) * tiles_y(C), tiles_x2(C) * tiles_y2(C)) * ((C.nz - 2 + kp - 1) / kp));
  return std::max(a, std::max(b, p));
}

// ----------------------------------------------------------------- host side

int gbf_split_alloc(gbf_domain* d) {
  const size_t n = gbf_geo(d->m).n;
  int s = GBF_OK;
  for (int b = 0; b < 2 && !s; b++) {
    s |= gbf_domain_alloc(d, (void**)&d->Pf[b], n * sizeof(float));
    s |= gbf_domain_alloc(d, (void**)&d->Sf[b], n * sizeof(float));
  }
  // FP64 masses or FP32 pairs: 8 bytes per cell and phase; FP32 defects: 4
  const int mb = gbf_mass_bytes(gbf_mass_rep(d->precision));
  if (!s) s |= gbf_domain_alloc(d, (void**)&d->M1, n * mb);
  if (!s) s |= gbf_domain_alloc(d, (void**)&d->M2, n * mb);
  // the defect form's water-mass part left out of the tiles' sums
  d->defect_k1v = 0.0;
  if (!s && gbf_is_defect(gbf_mass_rep(d->precision)))
    s |= gbf_defect_k1(d->m, d->cells.phi, d->cells.media, &d->defect_k1v, nullptr);  // after the cells' copies
  // per-block mass partials of the split step kernel
  if (!s) s |= gbf_domain_alloc(d, (void**)&d->split_partials, 2 * sizeof(double) * gbf_split_blocks(d->m, gbf_mass_rep(d->precision)));
  // the row table of the state conversions
  if (!s) s |= gbf_domain_alloc(d, (void**)&d->split_rows, sizeof(GbfRowConst) * (size_t)d->m.ny);
  if (!s) s |= gbf_split_fill_rows(d->m, d->split_rows, d->stream);
  // the Dirichlet patch's inflow, one FP32 pair per patch cell
  const int pn = gbf_patch_consts(d->m).n;
  if (!s && pn > 0) {  // zeroed: entries outside the interior are never written (nor used)
    s |= gbf_domain_alloc(d, (void**)&d->split_patch, sizeof(float2) * (size_t)pn * pn);
    if (!s) s |= gbf_cuda_check(cudaMemset(d->split_patch, 0, sizeof(float2) * (size_t)pn * pn), "gbf_split_alloc");
  }
  if (s) return GBF_ERR_NOMEM;
  // TMA plane loads: FP32 K and phi fields, no media table, rows of whole 16-byte units
  const gbf_model& m = d->m;
  if (d->cells.K && d->cells.phi && !d->cells.media && gbf_tma_eligible(m.nx, kPairTX)) {
    // boxes of the x-pair tile: halo planes {TX + 8, TY + 2}, interior rows {TX, TY}
    GbfTmaSet h;
    int e = GBF_OK;
    const int hx = kPairTX + 8, hy = kPairTY + 2;
    for (int b = 0; b < 2 && !e; b++) {
      e |= gbf_tma_encode_box(&h.dP[b], d->Pf[b], 4, m.nx, m.ny, m.nz, hx, hy);
      e |= gbf_tma_encode_box(&h.S[b], d->Sf[b], 4, m.nx, m.ny, m.nz, hx, hy);
    }
    if (!e) e |= gbf_tma_encode_box(&h.K, d->cells.K, 4, m.nx, m.ny, m.nz, hx, hy);
    if (!e) e |= gbf_tma_encode_box(&h.M1, d->M1, mb, m.nx, m.ny, m.nz, kPairTX, kPairTY);
    if (!e) e |= gbf_tma_encode_box(&h.M2, d->M2, mb, m.nx, m.ny, m.nz, kPairTX, kPairTY);
    if (!e) e |= gbf_tma_encode_box(&h.phi, d->cells.phi, 4, m.nx, m.ny, m.nz, kPairTX, kPairTY);
    if (!e && !gbf_domain_alloc(d, &d->tma, sizeof(GbfTmaSet))) {
      GBF_CUDA(cudaMemcpy(d->tma, &h, sizeof(GbfTmaSet), cudaMemcpyHostToDevice));
    } else {
      d->tma = nullptr;  // plain loads
      gbf_clear_status();
    }
  }
  return GBF_OK;
}

int gbf_defect_k1(const gbf_model& m, const float* phi_dev, const int* media_dev, double* k1v_host,
                  cudaStream_t st) {
  const int nrows = m.ny - 2;
  double* rows = nullptr;
  GBF_CUDA(cudaMallocAsync((void**)&rows, (nrows + 1) * sizeof(double), st));
  k_defect_k1_rows<<<nrows, 256, 0, st>>>(m, phi_dev, media_dev, rows);
  k_defect_k1_sum<<<1, 32, 0, st>>>(rows, nrows, m.h1 * m.h2 * m.h3, rows + nrows);
  GBF_CUDA(cudaGetLastError());
  GBF_CUDA(cudaMemcpyAsync(k1v_host, rows + nrows, sizeof(double), cudaMemcpyDeviceToHost, st));
  GBF_CUDA(cudaStreamSynchronize(st));
  GBF_CUDA(cudaFreeAsync(rows, st));
  return GBF_OK;
}

int gbf_split_fill_rows(const gbf_model& m, GbfRowConst* rows, cudaStream_t st) {
  k_split_rows<<<gbf_grid_for((size_t)m.ny, kThreads), kThreads, 0, st>>>(m, rows);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GBF_OK : gbf_cuda_check(e, "gbf_split_fill_rows");
}

int gbf_split_init_state(const gbf_model& m, const GbfRowConst* rows, const double* P_dev, const double* S_dev,
                         float* dPf, float* Sf, double* M1, double* M2, int mr, cudaStream_t st) {
  const size_t n = gbf_geo(m).n;
  k_split_init<<<gbf_grid_for(n, kThreads, 4), kThreads, 0, st>>>(m, rows, P_dev, S_dev, dPf, Sf, M1, M2, mr, 0, n);
  cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? GBF_OK : gbf_cuda_check(e, "gbf_split_init_state");
}

int gbf_split_upload(gbf_domain* d, const double* P1, const double* S2, cudaMemcpyKind kind) {
  const size_t n = gbf_geo(d->m).n, b = n * sizeof(double);
  const double *P = P1, *S = S2;
  double* tmp = nullptr;
  const double* mP = (const double*)gbf_mapped_host(P1);
  const double* mS = (const double*)gbf_mapped_host(S2);
  if (kind == cudaMemcpyHostToDevice && mP && mS) {  // page-locked: read in place
    P = mP;
    S = mS;
  } else if (kind == cudaMemcpyHostToDevice) {  // stage through device memory
    GBF_CUDA(cudaMallocAsync((void**)&tmp, 2 * b, d->stream));
    GBF_CUDA(cudaMemcpyAsync(tmp, P1, b, cudaMemcpyHostToDevice, d->stream));
    GBF_CUDA(cudaMemcpyAsync(tmp + n, S2, b, cudaMemcpyHostToDevice, d->stream));
    P = tmp;
    S = tmp + n;
  }
  d->cur = 0;
  k_split_init<<<gbf_grid_for(n, kThreads, 4), kThreads, 0, d->stream>>>(
      d->m, d->split_rows, P, S, d->Pf[0], d->Sf[0], d->M1, d->M2, gbf_mass_rep(d->precision), 0, n);
  GBF_CUDA(cudaGetLastError());
  // the next-state buffer's faces are rewritten every step; start them equal
  GBF_CUDA(cudaMemcpyAsync(d->Pf[1], d->Pf[0], n * sizeof(float), cudaMemcpyDeviceToDevice, d->stream));
  GBF_CUDA(cudaMemcpyAsync(d->Sf[1], d->Sf[0], n * sizeof(float), cudaMemcpyDeviceToDevice, d->stream));
  if (tmp) GBF_CUDA(cudaFreeAsync(tmp, d->stream));
  return GBF_OK;
}

int gbf_split_step(gbf_domain* d) {
  const int nxt = d->cur ^ 1;
  GbfSplitGrid G;
  G.dP = d->Pf[d->cur];
  G.S = d->Sf[d->cur];
  G.dPn = d->Pf[nxt];
  G.Sn = d->Sf[nxt];
  G.K = d->cells.K;
  G.phi = d->cells.phi;
  G.media = d->cells.media;
  G.M1 = d->M1;
  G.M2 = d->M2;
  G.mass_partials = nullptr;
  G.status = d->status;
  G.cfl_out = nullptr;
  G.patch_in = d->split_patch;
  double* mass_out = nullptr;
  if ((d->out_flags & GBF_OUT_MASS) && d->mass_hist && d->mass_count < d->mass_cap) {
    G.mass_partials = d->split_partials;
    mass_out = d->mass_hist + 2 * d->mass_count;
    if ((d->out_flags & GBF_OUT_CFL) && d->cfl_hist) G.cfl_out = d->cfl_hist + 2 * d->mass_count;
    d->mass_count++;
  }
  const GbfSplitConsts C = gbf_split_consts(d->m);
  int s = gbf_split_launch_domain(d->m, C, G, gbf_mass_rep(d->precision), mass_out, d->stream, &d->timer,
                                  (const GbfTmaSet*)d->tma, d->cur, d->defect_k1v);
  if (s) return s;
  d->cur = nxt;
  d->steps++;
  return GBF_OK;
}

int gbf_split_download(gbf_domain* d, int field, double* host) {
  const size_t n = gbf_geo(d->m).n, b = n * sizeof(double);
  if (field != GBF_FIELD_P1 && field != GBF_FIELD_S2)
    return gbf_fail(GBF_ERR_STATE, "split precision keeps P1 and S2 only");
  double* tmp = (double*)gbf_mapped_host(host);  // page-locked: written in place
  const bool staged = tmp == nullptr;
  if (staged) GBF_CUDA(cudaMallocAsync((void**)&tmp, b, d->stream));
  k_split_to_f64<<<gbf_grid_for(n, kThreads, 4), kThreads, 0, d->stream>>>(
      d->m, d->split_rows, d->Pf[d->cur], d->Sf[d->cur], field == GBF_FIELD_P1 ? tmp : nullptr,
      field == GBF_FIELD_S2 ? tmp : nullptr, 0, n);
  GBF_CUDA(cudaGetLastError());
  if (staged) {
    GBF_CUDA(cudaMemcpyAsync(host, tmp, b, cudaMemcpyDeviceToHost, d->stream));
    GBF_CUDA(cudaFreeAsync(tmp, d->stream));
  }
  GBF_CUDA(cudaStreamSynchronize(d->stream));
  return GBF_OK;
}

int gbf_split_state_to_f64(const gbf_model& m, const GbfRowConst* rows, const float* dPf, const float* Sf, double* P,
                           double* S, cudaStream_t st) {
  k_split_to_f64<<<gbf_grid_for(gbf_geo(m).n, kThreads, 4), kThreads, 0, st>>>(m, rows, dPf, Sf, P, S, 0,
                                                                                gbf_geo(m).n);
  GBF_CUDA(cudaGetLastError());
  return GBF_OK;
}

// One step of a grid from host FP64 arrays to host FP64 arrays, pipelined
// over slabs of planes (one k chunk layer of the step each): the copy engines
// move slab s + 1 in and slab s - 1 out while the compute stream converts slab
// s, steps the chunk layer of slab s - 1 (its tiles read the first plane of
// slab s), applies the boundary rules to its planes (they read nothing outside
// the slab but the start-of-step state) and converts it back. The state equals
// upload + step + download bit for bit; the phase masses sum the same cells in
// other partial blocks (within 1e-11 relative). Grids without a Dirichlet patch.
namespace {
int split_advance_host(gbf_domain* d, const double* P_in, const double* S_in, double* P_out, double* S_out) {
  const gbf_model& m = d->m;
  const GbfGeo g = gbf_geo(m);
  const size_t n = g.n, pl = g.pl;
  const int mr = gbf_mass_rep(d->precision);
  const GbfSplitConsts C = gbf_split_consts(m);
  const GbfTmaSet* maps = (const GbfTmaSet*)d->tma;
  const int kp = pipe_kchunk(C), ns = (C.nz - 2 + kp - 1) / kp;  // slabs = k chunks
  auto pa = [&](int q) { return q == 0 ? 0 : 1 + q * kp; };
  auto pb = [&](int q) { return q == ns - 1 ? C.nz : 1 + (q + 1) * kp; };
  if (!d->pipe_in) {
    GBF_CUDA(cudaStreamCreateWithFlags(&d->pipe_in, cudaStreamNonBlocking));
    GBF_CUDA(cudaStreamCreateWithFlags(&d->pipe_out, cudaStreamNonBlocking));
  }
  while ((int)d->pipe_ev.size() < 2 + 2 * ns) {
    cudaEvent_t e;
    GBF_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
    d->pipe_ev.push_back(e);
  }
  if (!d->pipe_stage && gbf_domain_alloc(d, (void**)&d->pipe_stage, 2 * sizeof(double) * n))
    return gbf_fail(GBF_ERR_NOMEM, "gbf_domain_advance_host");
  double *stP = d->pipe_stage, *stS = d->pipe_stage + n;
  cudaStream_t cs = d->stream;
  // the upload's resets (gbf_domain_upload), then everything on the stream so far first
  d->cur = 0;
  d->mass_count = 0;
  d->steps = 0;
  if (d->cfl_hist) GBF_CUDA(cudaMemsetAsync(d->cfl_hist, 0, 2 * sizeof(float) * (size_t)d->mass_cap, cs));
  GBF_CUDA(cudaMemsetAsync(d->status, 0, sizeof(unsigned), cs));
  GBF_CUDA(cudaEventRecord(d->pipe_ev[0], cs));
  GBF_CUDA(cudaStreamWaitEvent(d->pipe_in, d->pipe_ev[0], 0));
  GBF_CUDA(cudaStreamWaitEvent(d->pipe_out, d->pipe_ev[0], 0));
  for (int q = 0; q < ns; q++) {  // host -> device, every slab in order
    const size_t c0 = (size_t)pa(q) * pl, b = ((size_t)pb(q) * pl - c0) * sizeof(double);
    GBF_CUDA(cudaMemcpyAsync(stP + c0, P_in + c0, b, cudaMemcpyDefault, d->pipe_in));
    GBF_CUDA(cudaMemcpyAsync(stS + c0, S_in + c0, b, cudaMemcpyDefault, d->pipe_in));
    GBF_CUDA(cudaEventRecord(d->pipe_ev[2 + q], d->pipe_in));
  }
  GbfSplitGrid G;
  G.dP = d->Pf[0];
  G.S = d->Sf[0];
  G.dPn = d->Pf[1];
  G.Sn = d->Sf[1];
  G.K = d->cells.K;
  G.phi = d->cells.phi;
  G.media = d->cells.media;
  G.M1 = d->M1;
  G.M2 = d->M2;
  G.mass_partials = nullptr;
  G.status = d->status;
  G.cfl_out = nullptr;
  G.patch_in = nullptr;
  double* mass_out = nullptr;
  if ((d->out_flags & GBF_OUT_MASS) && d->mass_hist && d->mass_cap > 0) {
    G.mass_partials = d->split_partials;
    mass_out = d->mass_hist;
    if ((d->out_flags & GBF_OUT_CFL) && d->cfl_hist) G.cfl_out = d->cfl_hist;
    d->mass_count = 1;
  }
  const long long tiles = layer_tiles(C, maps);
  const size_t nb = maps ? gbf_boundary_count_no_xfaces(g) : gbf_boundary_count(g);
  for (int q = 0; q <= ns; q++) {
    if (q < ns) {  // slab q in: FP64 -> split state, both buffers
      const size_t c0 = (size_t)pa(q) * pl, c1 = (size_t)pb(q) * pl;
      GBF_CUDA(cudaStreamWaitEvent(cs, d->pipe_ev[2 + q], 0));
      k_split_init<<<gbf_grid_for(c1 - c0, kThreads, 4), kThreads, 0, cs>>>(m, d->split_rows, stP, stS, d->Pf[0],
                                                                          d->Sf[0], d->M1, d->M2, mr, c0, c1);
      GBF_CUDA(cudaMemcpyAsync(d->Pf[1] + c0, d->Pf[0] + c0, (c1 - c0) * sizeof(float), cudaMemcpyDeviceToDevice, cs));
      GBF_CUDA(cudaMemcpyAsync(d->Sf[1] + c0, d->Sf[0] + c0, (c1 - c0) * sizeof(float), cudaMemcpyDeviceToDevice, cs));
    }
    if (q > 0) {  // slab q - 1: its chunk layer of the step, its boundary cells, out
      const int r = q - 1;
      const size_t c0 = (size_t)pa(r) * pl, c1 = (size_t)pb(r) * pl;
      GbfSplitGrid Gr = G;
      if (Gr.mass_partials) Gr.mass_partials += 2 * (size_t)tiles * r;
      if (int s = launch_chunks(C, Gr, mr, maps, 0, cs, kp, r, 1)) return s;
      k_split_boundary<<<gbf_grid_for(nb, kThreads, 4), kThreads, 0, cs>>>(m, G, C.H, nb, pa(r), pb(r));
      k_split_to_f64<<<gbf_grid_for(c1 - c0, kThreads, 4), kThreads, 0, cs>>>(m, d->split_rows, d->Pf[1], d->Sf[1],
                                                                            stP, stS, c0, c1);
      GBF_CUDA(cudaGetLastError());
      GBF_CUDA(cudaEventRecord(d->pipe_ev[2 + ns + r], cs));
      GBF_CUDA(cudaStreamWaitEvent(d->pipe_out, d->pipe_ev[2 + ns + r], 0));
      const size_t b = (c1 - c0) * sizeof(double);
      GBF_CUDA(cudaMemcpyAsync(P_out + c0, stP + c0, b, cudaMemcpyDefault, d->pipe_out));
      GBF_CUDA(cudaMemcpyAsync(S_out + c0, stS + c0, b, cudaMemcpyDefault, d->pipe_out));
    }
  }
  if (mass_out)
    k_split_mass_tail<<<1, 256, 0, cs>>>(G.mass_partials, (int)(tiles * ns), mass_out,
                                         gbf_is_defect(mr) ? d->defect_k1v : 0.0);
  GBF_CUDA(cudaGetLastError());
  GBF_CUDA(cudaEventRecord(d->pipe_ev[1], d->pipe_out));
  GBF_CUDA(cudaStreamWaitEvent(cs, d->pipe_ev[1], 0));
  d->cur = 1;
  d->steps = 1;
  d->uploaded = true;
  GBF_CUDA(cudaStreamSynchronize(cs));
  return GBF_OK;
}
}  // namespace

int gbf_split_advance_host(gbf_domain* d, const double* P_in, const double* S_in, double* P_out, double* S_out) {
  const int s = split_advance_host(d, P_in, S_in, P_out, S_out);
  if (s) {  // an error part-way: no copy may still read or write the caller's arrays after the return
    if (d->pipe_in) cudaStreamSynchronize(d->pipe_in);
    if (d->pipe_out) cudaStreamSynchronize(d->pipe_out);
    cudaStreamSynchronize(d->stream);
  }
  return s;
}

int gbf_split_launches_per_step(gbf_domain* d) {
  return 2 + ((d->out_flags & GBF_OUT_MASS) ? 1 : 0) + (d->split_patch ? 1 : 0);
}

// ----------------------------------------------------------- diagnostics
// The bounded mbarrier wait of the TMA tiles, run on a barrier phase that
// never completes (arrival count 2, one arrival, no copy in flight): every
// thread must give up after `tries` rounds and the block reports
// GBF_DEV_TIMEOUT, as the tiles do when a plane never arrives.
namespace {
__global__ void k_diag_wait(unsigned tries, unsigned* status) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) {
    gbf_mbar_init(&bar, 2);
    gbf_mbar_fence_init();
  }
  __syncthreads();
  if (threadIdx.x == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(gbf_smem_u32(&bar)) : "memory");
  const bool ok = gbf_mbar_wait(&bar, 0u, tries);
  if (__syncthreads_or(!ok) && threadIdx.x == 0) atomicOr(status, GBF_DEV_TIMEOUT);
}
}  // namespace

extern "C" int gbf_diag_bounded_wait(unsigned tries, double* ms) {
  unsigned* st = nullptr;
  GBF_CUDA(cudaMalloc((void**)&st, sizeof(unsigned)));
  GBF_CUDA(cudaMemset(st, 0, sizeof(unsigned)));
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  cudaEventRecord(a, nullptr);
  k_diag_wait<<<1, 256>>>(tries, st);
  cudaEventRecord(b, nullptr);
  unsigned h = 0;
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpy(&h, st, sizeof(unsigned), cudaMemcpyDeviceToHost);
  float t = 0.f;
  if (e == cudaSuccess) cudaEventElapsedTime(&t, a, b);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  cudaFree(st);
  if (e != cudaSuccess) return gbf_cuda_check(e, "gbf_diag_bounded_wait");
  if (ms) *ms = t;
  return (h & GBF_DEV_TIMEOUT) ? gbf_fail(GBF_ERR_TIMEOUT, "bounded wait gave up (diagnostic)") : GBF_OK;
}
