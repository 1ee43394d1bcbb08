// gbf_ensemble.cu — batched ensembles: independent realizations of uneven
// grid sizes advanced together, one time step of every member per step.
//
// Split precision: one persistent kernel over a packed tile work list
// (member, x-tile, y-tile, k-range) of all members; CTAs take tiles from an
// atomic counter (dynamic balance of uneven members) and run the z-marching
// tile of gbf_split_tile.cuh with the member's constants copied to shared
// memory. Plain FP64: the two passes of gbf_f64_cell.cuh over packed chunk
// lists of all members' cells. Then one face pass over all members'
// boundary cells and one per-member phase-mass reduction. A step is a CUDA
// graph (counter reset, step, faces, masses), captured once per buffer parity.
//
// Tuning: the tile shape (one of the six compiled shapes of the enum below)
// and the k-range per CTA ("fusion depth": planes marched per tile pass) per
// member edge are picked by gbf_ensemble_autotune from timed trial steps.
#include <string.h>

#include <algorithm>
#include <map>
#include <vector>

#include "gbf_f64_cell.cuh"
#include "gbf_split_tile.cuh"

namespace {

struct EnsMember {
  gbf_model m;
  GbfDerived d;
  GbfSplitConsts C;
  gbf_cells cells;
  double* P[2];
  double* S[2];
  float* dPf[2];
  float* Sf[2];
  double *M1, *M2;
  double *L1, *L2, *ro1, *ro2, *lnSe;
  int part_begin, part_end;  // this member's slots in the partial-sum array
  double k1v;                // defect form: water-mass part left out of the tiles' sums (gbf_defect_k1)
  unsigned long long off;    // first cell of this member in the packed all-members layout
  // split forms under a Dirichlet patch: the pre-pass's constants and its FP64
  // inflow array (pc.n = 0, patch NULL: no patch)
  GbfPatchConsts pc;
  float2* patch;
  GbfRowConst* rows;  // split forms: the row constants of the state conversions (ny entries)
};

struct EnsChunk {
  int member;
  unsigned begin, end;
};

// Tile shapes (cells in x by rows); the last two are x-pair TMA tiles
// (split_tile_x2: two cells per thread, TMA staging only). 64x8 and 32x16
// pairs have the same shared memory (halo boxes {72, 10} and {40, 18}: 720
// elements each); the narrower one covers grids whose nx - 1 is just above a
// multiple of 64 with fewer idle lanes, and has the smaller halo (1.27x).
enum { kShape32x8 = 0, kShape64x4 = 1, kShape32x4 = 2, kShape64x8x2 = 3, kShape32x16x2 = 4, kShapeMixedx2 = 5,
       kShapes = 6 };
const int kShapeTX[kShapes] = {32, 64, 32, 64, 32, 32}, kShapeTY[kShapes] = {8, 4, 4, 8, 16, 16};
const bool kShapePairs[kShapes] = {false, false, false, true, true, true};
// The mixed shape's second tile: 48 x 10 cells, for the last 48 columns of a
// grid whose nx is 16 more than a multiple of 32 (nx >= 48).
constexpr int kWideTX = 48, kWideTY = 10;
bool mixed_wide_tail(int nx) { return nx >= 48 && nx % 32 > 0 && nx % 32 <= 16; }
constexpr int kChunkCells = 16384, kBoundaryChunk = 4096, kThreads = 256;

// ------------------------------------------------------------ split kernels

// Where a step's CFL numbers go (GBF_OUT_CFL): hist[step][member][2],
// step = *step_count (the mass history's step counter); NULL hist: off.
struct EnsCfl {
  const unsigned* step_count;
  float* hist;
  int n, cap;
};
__device__ __forceinline__ float* ens_cfl_slot(const EnsCfl& cfl, int member) {
  if (!cfl.hist) return nullptr;
  const unsigned step = *cfl.step_count;
  return step < (unsigned)cfl.cap ? cfl.hist + 2 * ((size_t)step * cfl.n + member) : nullptr;
}

template <int MR, int TX, int TY, bool TMA, bool CFL, bool PATCH>
__global__ void __launch_bounds__(TX * TY, 1024 / (TX * TY)) k_ens_split_step(const EnsMember* __restrict__ mem,
                                                                             const int4* __restrict__ tiles,
                                                                             const int* __restrict__ order,
                                                                             int ntiles, int cur,
                                                                             unsigned* counter, double* partials,
                                                                             unsigned* status,
                                                                             const GbfTmaSet* __restrict__ maps,
                                                                             const EnsCfl cfl) {
  __shared__ GbfSplitPlaneT<TX, TY, gbf_plane_pitch<TX, TMA>()> pl[TMA ? 3 : 2];
  __shared__ GbfSplitConsts Cs;
  __shared__ GbfSplitGrid Gs;
  __shared__ int s_tile;
  constexpr int NT = TX * TY;
  GbfRawRing<TX, TY, MR>* raw = nullptr;
  unsigned phases = 0;  // barrier parities of the stages, carried from tile to tile
  if constexpr (TMA) {
    __shared__ __align__(128) GbfRawRing<TX, TY, MR> ring;
    raw = &ring;
    if (threadIdx.x == 0) {
      for (int s = 0; s < kTmaStages; s++) gbf_mbar_init(&ring.bar[s], 1);
      for (int s = 0; s < GbfRawRing<TX, TY, MR>::RS; s++) gbf_mbar_init(&ring.mbar[s], 1);
      gbf_mbar_fence_init();
    }
    __syncthreads();
  }
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int t = s_tile;
    if (t >= ntiles) break;
    const int ti = order ? order[t] : t;  // list index (mass-partial slot)
    const int4 tl = tiles[ti];
    const EnsMember* me = mem + tl.x;
    {  // member constants to shared memory
      const int* src = reinterpret_cast<const int*>(&me->C);
      int* dst = reinterpret_cast<int*>(&Cs);
      for (int q = threadIdx.x; q < (int)(sizeof(GbfSplitConsts) / sizeof(int)); q += NT) dst[q] = src[q];
    }
    if (threadIdx.x == 0) {
      Gs.dP = me->dPf[cur];
      Gs.S = me->Sf[cur];
      Gs.dPn = me->dPf[cur ^ 1];
      Gs.Sn = me->Sf[cur ^ 1];
      Gs.K = me->cells.K;
      Gs.phi = me->cells.phi;
      Gs.media = me->cells.media;
      Gs.M1 = me->M1;
      Gs.M2 = me->M2;
      Gs.mass_partials = partials;
      Gs.status = status;
      Gs.cfl_out = CFL ? ens_cfl_slot(cfl, tl.x) : nullptr;
      if constexpr (PATCH) Gs.patch_in = me->patch;
    }
    __syncthreads();
    GbfSplitAcc<MR> acc;
    const bool ok = split_tile<MR, TX, TY, TMA, CFL, PATCH>(Cs, Gs, tl.y, tl.z, tl.w & 0xffff, tl.w >> 16, pl, acc, raw,
                                                TMA ? maps + tl.x : nullptr, cur, &phases);
    if (!ok) break;  // a plane wait gave up (status set); the whole CTA stops
    if (acc.bad) atomicOr(status, GBF_DEV_NONFINITE);
    if (partials) split_block_mass<MR, NT>(acc, Cs.V, partials + 2 * ti);
    if constexpr (CFL)
      if (Gs.cfl_out) split_block_cfl<NT>(acc.cfl1, acc.cfl2, Gs.cfl_out);
    __syncthreads();
  }
}

// Per tile: the member's constants to shared memory, its arrays to Gs.
template <int NT, bool CFL, bool PATCH>
__device__ __forceinline__ void ens_tile_setup(const EnsMember* me, int member, int cur, double* partials,
                                               unsigned* status, const EnsCfl& cfl, GbfSplitConsts& Cs,
                                               GbfSplitGrid& Gs) {
  const int* src = reinterpret_cast<const int*>(&me->C);
  int* dst = reinterpret_cast<int*>(&Cs);
  for (int q = threadIdx.x; q < (int)(sizeof(GbfSplitConsts) / sizeof(int)); q += NT) dst[q] = src[q];
  if (threadIdx.x == 0) {
    Gs.dP = me->dPf[cur];
    Gs.S = me->Sf[cur];
    Gs.dPn = me->dPf[cur ^ 1];
    Gs.Sn = me->Sf[cur ^ 1];
    Gs.K = me->cells.K;
    Gs.phi = me->cells.phi;
    Gs.media = me->cells.media;
    Gs.M1 = me->M1;
    Gs.M2 = me->M2;
    Gs.mass_partials = partials;
    Gs.status = status;
    Gs.cfl_out = CFL ? ens_cfl_slot(cfl, member) : nullptr;
    if constexpr (PATCH) Gs.patch_in = me->patch;
  }
}

// Tiles of the x-pair shapes carry their kind in bit 30 of the x origin:
// 0 the shape's own tile, 1 (mixed shape) a 48x10 tile.
constexpr int kTileKindShift = 30;
__host__ __device__ constexpr int tile_x0(int y) { return y & ((1 << kTileKindShift) - 1); }
__host__ __device__ constexpr int tile_kind(int y) { return y >> kTileKindShift; }

template <int MR, int TXC, int TY, bool CFL, bool PATCH>
__global__ void __launch_bounds__(TXC / 2 * TY, gbf_pair_ctas(MR) * 256 / (TXC / 2 * TY)) k_ens_split_step_x2(
    const EnsMember* __restrict__ mem, const int4* __restrict__ tiles, const int* __restrict__ order, int ntiles,
    int cur, unsigned* counter, double* partials, unsigned* status, const GbfTmaSet* __restrict__ maps,
    const EnsCfl cfl) {
  extern __shared__ __align__(128) unsigned char dyn[];
  using Cta = GbfPairCta<TXC, TY, MR>;
  Cta& cta = *reinterpret_cast<Cta*>(dyn);
  __shared__ GbfSplitConsts Cs;
  __shared__ GbfSplitGrid Gs;
  __shared__ int s_tile;
  constexpr int NT = TXC / 2 * TY;
  unsigned phases = 0;  // barrier parities of the stages, carried from tile to tile
  if (gbf_smem_u32(dyn) & 127u) {  // the TMA destinations need it; never expected to fire
    if (threadIdx.x == 0) atomicOr(status, GBF_DEV_TIMEOUT);
    return;
  }
  if (threadIdx.x == 0) gbf_pair_bars_init(cta.bars);
  __syncthreads();
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int t = s_tile;
    if (t >= ntiles) break;
    const int ti = order ? order[t] : t;  // list index (mass-partial slot)
    const int4 tl = tiles[ti];
    ens_tile_setup<NT, CFL, PATCH>(mem + tl.x, tl.x, cur, partials, status, cfl, Cs, Gs);
    __syncthreads();
    GbfSplitAcc<MR> acc;
    const bool ok = split_tile_x2<MR, TXC, TY, CFL, NT, PATCH>(Cs, Gs, tile_x0(tl.y), tl.z, tl.w & 0xffff,
                                                              tl.w >> 16, cta.bars, cta.body, acc, maps + tl.x, cur,
                                                              &phases);
    if (!ok) break;
    if (acc.bad) atomicOr(status, GBF_DEV_NONFINITE);
    if (partials) split_block_mass<MR, NT>(acc, Cs.V, partials + 2 * ti);
    if constexpr (CFL)
      if (Gs.cfl_out) split_block_cfl<NT>(acc.cfl1, acc.cfl2, Gs.cfl_out);
    __syncthreads();
  }
}

// The mixed x-pair shape: 32x16 tiles, and 48x10 tiles for the last 48
// columns of members whose nx is 16 more than a multiple of 32 (fewer idle
// lanes than a half-empty 32-wide tile). One set of barriers serves both
// shapes' rings, which share the shared memory (a union); `maps` holds two
// sets per member (32x16, 48x10 boxes).
template <int MR, bool CFL, bool PATCH>
__global__ void __launch_bounds__(256, gbf_pair_ctas(MR)) k_ens_split_step_x2m(
    const EnsMember* __restrict__ mem, const int4* __restrict__ tiles, const int* __restrict__ order, int ntiles,
    int cur, unsigned* counter, double* partials, unsigned* status, const GbfTmaSet* __restrict__ maps,
    const EnsCfl cfl) {
  extern __shared__ __align__(128) unsigned char dyn[];
  using Cta = GbfPairCtaMixed<MR>;
  Cta& cta = *reinterpret_cast<Cta*>(dyn);
  __shared__ GbfSplitConsts Cs;
  __shared__ GbfSplitGrid Gs;
  __shared__ int s_tile;
  constexpr int NT = 256;
  unsigned phases = 0;
  if (gbf_smem_u32(dyn) & 127u) {  // the TMA destinations need it; never expected to fire
    if (threadIdx.x == 0) atomicOr(status, GBF_DEV_TIMEOUT);
    return;
  }
  if (threadIdx.x == 0) gbf_pair_bars_init(cta.bars);
  __syncthreads();
  for (;;) {
    if (threadIdx.x == 0) s_tile = (int)atomicAdd(counter, 1u);
    __syncthreads();
    const int t = s_tile;
    if (t >= ntiles) break;
    const int ti = order ? order[t] : t;
    const int4 tl = tiles[ti];
    ens_tile_setup<NT, CFL, PATCH>(mem + tl.x, tl.x, cur, partials, status, cfl, Cs, Gs);
    __syncthreads();
    GbfSplitAcc<MR> acc;
    const int x0 = tile_x0(tl.y), k0 = tl.w & 0xffff, k1 = tl.w >> 16;
    const bool ok = tile_kind(tl.y)
                        ? split_tile_x2<MR, 48, 10, CFL, NT, PATCH>(Cs, Gs, x0, tl.z, k0, k1, cta.bars, cta.b, acc,
                                                                    maps + 2 * tl.x + 1, cur, &phases)
                        : split_tile_x2<MR, 32, 16, CFL, NT, PATCH>(Cs, Gs, x0, tl.z, k0, k1, cta.bars, cta.a, acc,
                                                                    maps + 2 * tl.x, cur, &phases);
    if (!ok) break;
    if (acc.bad) atomicOr(status, GBF_DEV_NONFINITE);
    if (partials) split_block_mass<MR, NT>(acc, Cs.V, partials + 2 * ti);
    if constexpr (CFL)
      if (Gs.cfl_out) split_block_cfl<NT>(acc.cfl1, acc.cfl2, Gs.cfl_out);
    // the next tile's copies may land where this tile's threads wrote (the
    // other shape's plane buffers): order the generic writes before them
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kThreads) k_ens_split_boundary(const EnsMember* __restrict__ mem,
                                                                 const EnsChunk* __restrict__ chunks, int cur) {
  const EnsChunk ch = chunks[blockIdx.x];
  const EnsMember* me = mem + ch.member;
  const gbf_model& m = me->m;
  const GbfGeo g = gbf_geo(m);
  const float* dP = me->dPf[cur];
  const float* S = me->Sf[cur];
  float* dPn = me->dPf[cur ^ 1];
  float* Sn = me->Sf[cur ^ 1];
  const float H = me->C.H;
  for (unsigned t = ch.begin + threadIdx.x; t < ch.end; t += blockDim.x) {
    int i, j, k;
    gbf_boundary_cell(g, t, i, j, k);
    const size_t c = gbf_idx(g, i, j, k);
    Sn[c] = gbf_sweep_S<float>(m, g, Sn, S, i, j, k);
    dPn[c] = gbf_split_sweep_dP(m, g, dPn, dP, i, j, k, H);
  }
}

// The face pass after the x-pair tiles: each block takes kThreads / 32 row
// segments of one member (gbf_split_face_segment), one per warp.
__global__ void __launch_bounds__(kThreads) k_ens_split_faces(const EnsMember* __restrict__ mem,
                                                              const EnsChunk* __restrict__ chunks, int cur) {
  const EnsChunk ch = chunks[blockIdx.x];
  const unsigned w = ch.begin + (threadIdx.x >> 5);
  if (w >= ch.end) return;
  const EnsMember* me = mem + ch.member;
  const gbf_model& m = me->m;
  const GbfGeo g = gbf_geo(m);
  const int segs = (m.nx + kFaceSeg - 1) / kFaceSeg;
  const int r = (int)w / segs, seg = (int)w - r * segs;
  int j, k;
  gbf_face_row(g, r, j, k);
  gbf_split_face_segment(m, g, me->dPf[cur], me->Sf[cur], me->dPf[cur ^ 1], me->Sf[cur ^ 1], me->C.H, j, k,
                         seg * kFaceSeg, (int)(threadIdx.x & 31));
}

// ------------------------------------------------------------- FP64 kernels

__device__ __forceinline__ GbfF64Step ens_f64_step(const EnsMember& me, int cur) {
  GbfF64Step s = {};
  s.P = me.P[cur];
  s.S = me.S[cur];
  s.Pn = me.P[cur ^ 1];
  s.Sn = me.S[cur ^ 1];
  s.L1 = me.L1; s.L2 = me.L2; s.ro1 = me.ro1; s.ro2 = me.ro2; s.lnSe = me.lnSe;
  return s;
}

__global__ void __launch_bounds__(kThreads) k_ens_f64_props(const EnsMember* __restrict__ mem,
                                                            const EnsChunk* __restrict__ chunks, int cur) {
  __shared__ EnsMember me;
  const EnsChunk ch = chunks[blockIdx.x];
  {
    const int* src = reinterpret_cast<const int*>(mem + ch.member);
    int* dst = reinterpret_cast<int*>(&me);
    for (int q = threadIdx.x; q < (int)(sizeof(EnsMember) / sizeof(int)); q += blockDim.x) dst[q] = src[q];
  }
  __syncthreads();
  const GbfGeo g = gbf_geo(me.m);
  const GbfF64Step s = ens_f64_step(me, cur);
  for (unsigned c = ch.begin + threadIdx.x; c < ch.end; c += blockDim.x) gbf_f64_props_cell(me.m, me.d, me.cells, s, 0, g, c);
}

__global__ void __launch_bounds__(kThreads) k_ens_f64_flux_newton(const EnsMember* __restrict__ mem,
                                                                  const EnsChunk* __restrict__ chunks, int cur,
                                                                  double* partials, unsigned* status) {
  __shared__ EnsMember me;
  const EnsChunk ch = chunks[blockIdx.x];
  {
    const int* src = reinterpret_cast<const int*>(mem + ch.member);
    int* dst = reinterpret_cast<int*>(&me);
    for (int q = threadIdx.x; q < (int)(sizeof(EnsMember) / sizeof(int)); q += blockDim.x) dst[q] = src[q];
  }
  __syncthreads();
  const GbfGeo g = gbf_geo(me.m);
  const GbfF64Step s = ens_f64_step(me, cur);
  const unsigned ix = g.nx - 2, iy = g.ny - 2;
  double m1 = 0., m2 = 0.;
  unsigned bad = 0;
  for (unsigned t = ch.begin + threadIdx.x; t < ch.end; t += blockDim.x) {
    const int i = 1 + (int)(t % ix), j = 1 + (int)((t / ix) % iy), k = 1 + (int)(t / (ix * iy));
    gbf_f64_flux_newton_cell(me.m, me.d, me.cells, s, g, i, j, k, m1, m2, bad);
  }
  if (bad) atomicOr(status, GBF_DEV_NONFINITE);
  if (partials) gbf_block_sum2<kThreads>(m1, m2, me.d.V, partials + 2 * blockIdx.x);
}

__global__ void __launch_bounds__(kThreads) k_ens_f64_boundary(const EnsMember* __restrict__ mem,
                                                               const EnsChunk* __restrict__ chunks, int cur) {
  const EnsChunk ch = chunks[blockIdx.x];
  const EnsMember& me = mem[ch.member];
  const GbfGeo g = gbf_geo(me.m);
  const GbfF64Step s = ens_f64_step(me, cur);
  for (unsigned t = ch.begin + threadIdx.x; t < ch.end; t += blockDim.x) gbf_f64_boundary_cell(me.m, s, g, t);
}

// Per-member phase masses of this step: one block per member sums its
// partials in a fixed order into hist[step][member][2] (step from *count).
__global__ void k_ens_mass_tail(const EnsMember* __restrict__ mem, const double* partials, double* hist,
                                unsigned* count, int nmem, int cap) {
  __shared__ double red[2][256];
  const EnsMember& me = mem[blockIdx.x];
  double a = 0., b = 0.;
  for (int q = me.part_begin + threadIdx.x; q < me.part_end; q += blockDim.x) {
    a += partials[2 * q];
    b += partials[2 * q + 1];
  }
  red[0][threadIdx.x] = a;
  red[1][threadIdx.x] = b;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) { red[0][threadIdx.x] += red[0][threadIdx.x + o]; red[1][threadIdx.x] += red[1][threadIdx.x + o]; }
    __syncthreads();
  }
  const unsigned step = *count;
  if (threadIdx.x == 0 && step < (unsigned)cap) {
    hist[2 * ((size_t)step * nmem + blockIdx.x)] = red[0][0] + me.k1v;
    hist[2 * ((size_t)step * nmem + blockIdx.x) + 1] = red[1][0];
  }
}
__global__ void k_ens_count(unsigned* count) { atomicAdd(count, 1u); }

// The step's pre-pass for split members under a Dirichlet patch
// (gbf_split_patch_cell), one block per member of [r0, r0 + gridDim.x).
__global__ void __launch_bounds__(64) k_ens_split_patch(const EnsMember* __restrict__ mem, int r0, int cur) {
  const EnsMember& me = mem[r0 + blockIdx.x];
  if (!me.patch) return;
  GbfSplitGrid G = {};
  G.dP = me.dPf[cur];
  G.S = me.Sf[cur];
  G.K = me.cells.K;
  G.phi = me.cells.phi;
  G.media = me.cells.media;
  G.patch_in = me.patch;
  for (int t = threadIdx.x; t < me.pc.n * me.pc.n; t += blockDim.x) gbf_split_patch_cell(me.C, me.pc, G, t);
}

// Packed all-members FP64 state (staging) -> every member's current buffer
// (and the next buffer's faces, which the next step rewrites), one chunk
// (member, cell range) per block.
__global__ void __launch_bounds__(kThreads) k_ens_load(const EnsMember* __restrict__ mem,
                                                       const EnsChunk* __restrict__ chunks, int cur,
                                                       const double* __restrict__ P_all,
                                                       const double* __restrict__ S_all, int precision) {
  const EnsChunk ch = chunks[blockIdx.x];
  const EnsMember& me = mem[ch.member];
  const gbf_model& m = me.m;
  for (unsigned c = ch.begin + threadIdx.x; c < ch.end; c += blockDim.x) {
    const double p = P_all[me.off + c], s = S_all[me.off + c];
    if (precision == GBF_PREC_F64) {
      me.P[cur][c] = p;
      me.S[cur][c] = s;
    } else {
      const int j = (int)((c / (unsigned)m.nx) % (unsigned)m.ny);
      float dPf, Sf;
      gbf_split_init_cell(m, p, s, me.rows[j], dPf, Sf, me.M1, me.M2, c, gbf_mass_rep(precision));
      me.dPf[cur][c] = dPf;
      me.Sf[cur][c] = Sf;
      me.dPf[cur ^ 1][c] = dPf;
      me.Sf[cur ^ 1][c] = Sf;
    }
  }
}

// The row-constant tables of the split members, one block per member.
__global__ void k_ens_rows(const EnsMember* __restrict__ mem) {
  const EnsMember& me = mem[blockIdx.x];
  if (!me.rows) return;
  for (int j = threadIdx.x; j < me.m.ny; j += blockDim.x) me.rows[j] = gbf_row_const(me.m, j);
}

// Every member's current state -> packed all-members FP64 arrays.
__global__ void __launch_bounds__(kThreads) k_ens_store(const EnsMember* __restrict__ mem,
                                                        const EnsChunk* __restrict__ chunks, int cur,
                                                        double* __restrict__ P_all, double* __restrict__ S_all,
                                                        int precision) {
  const EnsChunk ch = chunks[blockIdx.x];
  const EnsMember& me = mem[ch.member];
  const gbf_model& m = me.m;
  for (unsigned c = ch.begin + threadIdx.x; c < ch.end; c += blockDim.x) {
    if (precision == GBF_PREC_F64) {
      P_all[me.off + c] = me.P[cur][c];
      S_all[me.off + c] = me.S[cur][c];
    } else {
      const int j = (int)((c / (unsigned)m.nx) % (unsigned)m.ny);
      P_all[me.off + c] = me.rows[j].phs + (double)me.dPf[cur][c];
      S_all[me.off + c] = (double)me.Sf[cur][c];
    }
  }
}

}  // namespace

// ----------------------------------------------------------------- object

struct gbf_ensemble {
  int n = 0;
  int precision = GBF_PREC_SPLIT_DF;
  std::vector<gbf_model> models;
  std::vector<EnsMember> h_mem;
  EnsMember* d_mem = nullptr;
  std::vector<int4> tiles;
  int4* d_tiles = nullptr;
  int* d_order = nullptr;  // whole-ensemble processing order of the tiles: longest k ranges first
  std::vector<EnsChunk> props, flux, bnd, all;
  EnsChunk *d_props = nullptr, *d_flux = nullptr, *d_bnd = nullptr, *d_all = nullptr;
  double* d_stage = nullptr;  // packed FP64 P, S of all members (whole-ensemble transfers)
  GbfTmaSet* d_maps = nullptr;  // per-member TMA plane maps of the current tile shape (NULL: plain loads)
  int nparts = 0;
  double* d_partials = nullptr;
  unsigned *d_counter = nullptr, *d_status = nullptr, *d_mass_count = nullptr;
  double* d_mass_hist = nullptr;
  float* d_cfl_hist = nullptr;  // [mass_cap][n][2] (GBF_OUT_CFL)
  int mass_cap = 0;
  int out_flags = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int cur = 0;
  bool any_patch = false;  // a split member under a Dirichlet patch: PATCH tiles and the step's pre-pass
  int shape = kShape32x8;
  std::map<int, int> kchunk_by_edge;  // fusion depth per member edge (0 = default rule)
  int persistent_blocks = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};
  GbfTimer timer;
  std::vector<void*> owned;
  long long steps = 0, cells = 0;
  bool uploaded_all = false;
  // first entry of each member in the packed lists (n + 1 rows; row n = totals)
  struct ListStarts { int tiles, props, flux, bnd, all; };
  std::vector<ListStarts> starts;
  // host-resident pipeline (gbf_ensemble_advance_host): copy streams, events,
  // one tile counter per member group
  cudaStream_t s_in = nullptr, s_out = nullptr;
  std::vector<cudaEvent_t> ev;  // [0] start, [1] end, then 2 per group
  unsigned* d_gcounter = nullptr;
  int pipe_groups = 0;  // requested group count (0: automatic)
};

namespace {

int ens_alloc(gbf_ensemble* e, void** p, size_t bytes) {
  cudaError_t r = cudaMalloc(p, bytes ? bytes : 16);
  if (r != cudaSuccess) {
    *p = nullptr;
    return gbf_cuda_check(r, "gbf_ensemble alloc");
  }
  e->owned.push_back(*p);
  return GBF_OK;
}

void drop_graphs(gbf_ensemble* e) {
  for (auto& g : e->graph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

int default_kchunk(const gbf_model& m) { return std::max(1, m.nz - 2); }

int kchunk_for(const gbf_ensemble* e, const gbf_model& m) {
  auto it = e->kchunk_by_edge.find(m.nx);
  int kc = (it != e->kchunk_by_edge.end() && it->second > 0) ? it->second : default_kchunk(m);
  return std::min(kc, m.nz - 2);
}

// Whether every member can stage its planes by TMA for tiles TX cells wide:
// FP32 K and phi fields, no media table, rows of whole 16-byte units.
bool tma_possible(const gbf_ensemble* e, int TX) {
  for (int r = 0; r < e->n; r++) {
    const EnsMember& me = e->h_mem[r];
    if (!(me.cells.K && me.cells.phi && !me.cells.media && gbf_tma_eligible(e->models[r].nx, TX))) return false;
  }
  return true;
}

// Packed work lists of the current tuning.
int build_lists(gbf_ensemble* e) {
  e->tiles.clear();
  e->props.clear();
  e->flux.clear();
  e->bnd.clear();
  e->all.clear();
  const bool split = e->precision != GBF_PREC_F64;
  const int TX = kShapeTX[e->shape], TY = kShapeTY[e->shape];
  e->starts.assign(e->n + 1, {});
  auto mark = [&](int r) {
    e->starts[r] = {(int)e->tiles.size(), (int)e->props.size(), (int)e->flux.size(), (int)e->bnd.size(),
                    (int)e->all.size()};
  };
  for (int r = 0; r < e->n; r++) {
    const gbf_model& m = e->models[r];
    const GbfGeo g = gbf_geo(m);
    EnsMember& me = e->h_mem[r];
    mark(r);
    if (split) {
      me.part_begin = (int)e->tiles.size();
      const int kc = kchunk_for(e, m);
      // tiles start at i0 = 1 + t TX, or at x0 = t TX for the x-pair shapes;
      // the mixed shape ends a row of 32-wide tiles with a 48x10 tile where
      // that covers the last columns with fewer idle lanes
      const int first = kShapePairs[e->shape] ? 0 : 1;
      const bool wide = e->shape == kShapeMixedx2 && mixed_wide_tail(m.nx);
      const int x_end = wide ? (m.nx / 32 - 1) * 32 : m.nx - 1;  // end of the TX-wide tiles' origins
      for (int k0 = 1; k0 < m.nz - 1; k0 += kc) {
        const int k1 = std::min(k0 + kc, m.nz - 1);
        for (int j0 = 1; j0 < m.ny - 1; j0 += TY)
          for (int i0 = first; i0 < x_end; i0 += TX) e->tiles.push_back(make_int4(r, i0, j0, k0 | (k1 << 16)));
        if (wide)
          for (int j0 = 1; j0 < m.ny - 1; j0 += kWideTY)
            e->tiles.push_back(make_int4(r, x_end | (1 << kTileKindShift), j0, k0 | (k1 << 16)));
      }
      me.part_end = (int)e->tiles.size();
    } else {
      for (unsigned b = 0; b < g.n; b += kChunkCells) e->props.push_back({r, b, (unsigned)std::min<size_t>(g.n, b + kChunkCells)});
      const size_t nint = (size_t)(m.nx - 2) * (m.ny - 2) * (m.nz - 2);
      me.part_begin = (int)e->flux.size();
      for (unsigned b = 0; b < nint; b += kChunkCells) e->flux.push_back({r, b, (unsigned)std::min<size_t>(nint, b + kChunkCells)});
      me.part_end = (int)e->flux.size();
    }
    if (split && kShapePairs[e->shape]) {
      // the x-pair tile writes the x faces itself; the face pass takes the
      // other face cells as row segments, kThreads / 32 per block
      const unsigned items = (unsigned)(gbf_face_rows(g) * ((m.nx + kFaceSeg - 1) / kFaceSeg));
      for (unsigned b = 0; b < items; b += kThreads / 32) e->bnd.push_back({r, b, std::min(items, b + kThreads / 32)});
    } else {
      const size_t nb = gbf_boundary_count(g);
      for (unsigned b = 0; b < nb; b += kBoundaryChunk) e->bnd.push_back({r, b, (unsigned)std::min<size_t>(nb, b + kBoundaryChunk)});
    }
    for (unsigned b = 0; b < g.n; b += kChunkCells) e->all.push_back({r, b, (unsigned)std::min<size_t>(g.n, b + kChunkCells)});
  }
  mark(e->n);
  // device copies (reallocated when they grow)
  auto upload = [&](void** dptr, const void* src, size_t bytes) -> int {
    if (*dptr) {
      auto it = std::find(e->owned.begin(), e->owned.end(), *dptr);
      if (it != e->owned.end()) e->owned.erase(it);
      cudaFree(*dptr);
      *dptr = nullptr;
    }
    if (int s = ens_alloc(e, dptr, bytes)) return s;
    GBF_CUDA(cudaMemcpy(*dptr, src, bytes, cudaMemcpyHostToDevice));
    return GBF_OK;
  };
  int s = GBF_OK;
  if (split) {
    s |= upload((void**)&e->d_tiles, e->tiles.data(), e->tiles.size() * sizeof(int4));
    e->nparts = (int)e->tiles.size();
    // longest-processing-time-first order for the whole-ensemble step: the
    // persistent CTAs end on the short tiles, which shortens the tail
    std::vector<int> order(e->tiles.size());
    for (size_t q = 0; q < order.size(); q++) order[q] = (int)q;
    auto planes = [&](int q) { return (e->tiles[q].w >> 16) - (e->tiles[q].w & 0xffff); };
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return planes(a) > planes(b); });
    s |= upload((void**)&e->d_order, order.data(), order.size() * sizeof(int));
  } else {
    s |= upload((void**)&e->d_props, e->props.data(), e->props.size() * sizeof(EnsChunk));
    s |= upload((void**)&e->d_flux, e->flux.data(), e->flux.size() * sizeof(EnsChunk));
    e->nparts = (int)e->flux.size();
  }
  s |= upload((void**)&e->d_bnd, e->bnd.data(), e->bnd.size() * sizeof(EnsChunk));
  s |= upload((void**)&e->d_all, e->all.data(), e->all.size() * sizeof(EnsChunk));
  s |= upload((void**)&e->d_partials, std::vector<double>(2 * (size_t)std::max(1, e->nparts), 0.0).data(),
              2 * sizeof(double) * std::max(1, e->nparts));
  s |= upload((void**)&e->d_mem, e->h_mem.data(), e->h_mem.size() * sizeof(EnsMember));
  // TMA maps for the tile shape, when every member qualifies (FP32 K and phi
  // fields, no media table, rows of whole 16-byte units)
  if (e->d_maps) {
    auto it = std::find(e->owned.begin(), e->owned.end(), (void*)e->d_maps);
    if (it != e->owned.end()) e->owned.erase(it);
    cudaFree(e->d_maps);
    e->d_maps = nullptr;
  }
  const bool tma = split && tma_possible(e, TX);
  if (kShapePairs[e->shape] && !tma) return gbf_fail(GBF_ERR_ARG, "the x-pair tile needs TMA staging");
  const int mb = gbf_mass_bytes(gbf_mass_rep(e->precision));  // bytes of a mass element
  if (tma && !s) {
    const bool mixed = e->shape == kShapeMixedx2;
    std::vector<GbfTmaSet> maps(mixed ? 2 * e->n : e->n);
    int enc = GBF_OK;
    // split_tile_x2 boxes: halo {tx + 8, ty + 2}, rows {tx, ty}
    auto pair_maps = [&](GbfTmaSet& q, const EnsMember& me, const gbf_model& m, int tx, int ty) {
      for (int b = 0; b < 2; b++) {
        enc |= gbf_tma_encode_box(&q.dP[b], me.dPf[b], 4, m.nx, m.ny, m.nz, tx + 8, ty + 2);
        enc |= gbf_tma_encode_box(&q.S[b], me.Sf[b], 4, m.nx, m.ny, m.nz, tx + 8, ty + 2);
      }
      enc |= gbf_tma_encode_box(&q.K, me.cells.K, 4, m.nx, m.ny, m.nz, tx + 8, ty + 2);
      enc |= gbf_tma_encode_box(&q.M1, me.M1, mb, m.nx, m.ny, m.nz, tx, ty);
      enc |= gbf_tma_encode_box(&q.M2, me.M2, mb, m.nx, m.ny, m.nz, tx, ty);
      enc |= gbf_tma_encode_box(&q.phi, me.cells.phi, 4, m.nx, m.ny, m.nz, tx, ty);
    };
    for (int r = 0; r < e->n && !enc; r++) {
      const EnsMember& me = e->h_mem[r];
      const gbf_model& m = e->models[r];
      if (mixed) {  // [2 r]: 32x16 boxes, [2 r + 1]: 48x10 boxes
        pair_maps(maps[2 * r], me, m, TX, TY);
        pair_maps(maps[2 * r + 1], me, m, kWideTX, kWideTY);
        continue;
      }
      if (kShapePairs[e->shape]) {
        pair_maps(maps[r], me, m, TX, TY);
        continue;
      }
      for (int b = 0; b < 2; b++) {
        enc |= gbf_tma_encode_plane(&maps[r].dP[b], me.dPf[b], m.nx, m.ny, m.nz, TX, TY);
        enc |= gbf_tma_encode_plane(&maps[r].S[b], me.Sf[b], m.nx, m.ny, m.nz, TX, TY);
      }
      enc |= gbf_tma_encode_plane(&maps[r].K, me.cells.K, m.nx, m.ny, m.nz, TX, TY);
      enc |= gbf_tma_encode_rows(&maps[r].M1, me.M1, mb, m.nx, m.ny, m.nz, TX, TY);
      enc |= gbf_tma_encode_rows(&maps[r].M2, me.M2, mb, m.nx, m.ny, m.nz, TX, TY);
      enc |= gbf_tma_encode_rows(&maps[r].phi, me.cells.phi, 4, m.nx, m.ny, m.nz, TX, TY);
    }
    if (!enc)
      s |= upload((void**)&e->d_maps, maps.data(), maps.size() * sizeof(GbfTmaSet));
    else
      gbf_clear_status();  // plain loads
  }
  drop_graphs(e);
  return s ? GBF_ERR_CUDA : GBF_OK;
}

// Tiles [t0, t0 + nt) of the packed list, buffer parity `cur`; the CTAs
// take tiles from `counter` (zeroed beforehand on the same stream).
struct TileRange {
  int t0, nt, cur;
  unsigned* counter;
  const int* order;  // processing order of tiles [0, nt) (absolute indices; t0 = 0), or NULL: list order
};

EnsCfl ens_cfl(const gbf_ensemble* e) {
  const bool on = (e->out_flags & GBF_OUT_CFL) && (e->out_flags & GBF_OUT_MASS) && e->d_cfl_hist;
  return {e->d_mass_count, on ? e->d_cfl_hist : nullptr, e->n, e->mass_cap};
}

template <int MR, int TX, int TY, bool PATCH>
int launch_split_step_t(gbf_ensemble* e, double* partials, cudaStream_t st, const TileRange& tr) {
  const bool tma = e->d_maps != nullptr, cfl = partials && ens_cfl(e).hist;
  auto kern = tma ? (cfl ? k_ens_split_step<MR, TX, TY, true, true, PATCH> : k_ens_split_step<MR, TX, TY, true, false, PATCH>)
                  : (cfl ? k_ens_split_step<MR, TX, TY, false, true, PATCH>
                         : k_ens_split_step<MR, TX, TY, false, false, PATCH>);
  int per_sm = 0;
  GBF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TX * TY, 0));
  const int blocks = std::max(1, std::min(tr.nt, per_sm * gbf_num_sms()));
  e->persistent_blocks = blocks;
  kern<<<blocks, TX * TY, 0, st>>>(e->d_mem, e->d_tiles + tr.t0, tr.order, tr.nt, tr.cur, tr.counter,
                                    partials ? partials + 2 * (size_t)tr.t0 : nullptr, e->d_status, e->d_maps,
                                    ens_cfl(e));
  return GBF_OK;
}

template <int MR, int TXC, int TY, bool PATCH>
int launch_split_step_x2(gbf_ensemble* e, double* partials, cudaStream_t st, const TileRange& tr) {
  if (!e->d_maps) return gbf_fail(GBF_ERR_STATE, "x-pair tile without TMA maps");
  auto kern = (partials && ens_cfl(e).hist) ? k_ens_split_step_x2<MR, TXC, TY, true, PATCH>
                                            : k_ens_split_step_x2<MR, TXC, TY, false, PATCH>;
  const int bytes = (int)sizeof(GbfPairCta<TXC, TY, MR>);
  GBF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  int per_sm = 0;
  GBF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, TXC / 2 * TY, bytes));
  const int blocks = std::max(1, std::min(tr.nt, std::max(1, per_sm) * gbf_num_sms()));
  e->persistent_blocks = blocks;
  kern<<<blocks, TXC / 2 * TY, bytes, st>>>(e->d_mem, e->d_tiles + tr.t0, tr.order, tr.nt, tr.cur, tr.counter,
                                             partials ? partials + 2 * (size_t)tr.t0 : nullptr, e->d_status,
                                             e->d_maps, ens_cfl(e));
  return GBF_OK;
}

template <int MR, bool PATCH>
int launch_split_step_x2m(gbf_ensemble* e, double* partials, cudaStream_t st, const TileRange& tr) {
  if (!e->d_maps) return gbf_fail(GBF_ERR_STATE, "x-pair tile without TMA maps");
  auto kern = (partials && ens_cfl(e).hist) ? k_ens_split_step_x2m<MR, true, PATCH> : k_ens_split_step_x2m<MR, false, PATCH>;
  const int bytes = (int)sizeof(GbfPairCtaMixed<MR>);
  GBF_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
  int per_sm = 0;
  GBF_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, bytes));
  const int blocks = std::max(1, std::min(tr.nt, std::max(1, per_sm) * gbf_num_sms()));
  e->persistent_blocks = blocks;
  kern<<<blocks, 256, bytes, st>>>(e->d_mem, e->d_tiles + tr.t0, tr.order, tr.nt, tr.cur, tr.counter,
                                   partials ? partials + 2 * (size_t)tr.t0 : nullptr, e->d_status, e->d_maps,
                                   ens_cfl(e));
  return GBF_OK;
}

template <int MR, bool PATCH>
int launch_split_shape(gbf_ensemble* e, double* partials, cudaStream_t st, const TileRange& tr) {
  switch (e->shape) {
    case kShapeMixedx2: return launch_split_step_x2m<MR, PATCH>(e, partials, st, tr);
    case kShape64x8x2: return launch_split_step_x2<MR, 64, 8, PATCH>(e, partials, st, tr);
    case kShape32x16x2: return launch_split_step_x2<MR, 32, 16, PATCH>(e, partials, st, tr);
    case kShape64x4: return launch_split_step_t<MR, 64, 4, PATCH>(e, partials, st, tr);
    case kShape32x4: return launch_split_step_t<MR, 32, 4, PATCH>(e, partials, st, tr);
    default: return launch_split_step_t<MR, 32, 8, PATCH>(e, partials, st, tr);
  }
}

// Ensembles with a member under a Dirichlet patch run the PATCH tiles.
template <int MR>
int launch_split_form(gbf_ensemble* e, double* partials, cudaStream_t st, const TileRange& tr) {
  return e->any_patch ? launch_split_shape<MR, true>(e, partials, st, tr)
                      : launch_split_shape<MR, false>(e, partials, st, tr);
}

int launch_split_step(gbf_ensemble* e, double* partials, cudaStream_t st, const TileRange& tr) {
  switch (gbf_mass_rep(e->precision)) {
    case kMassDefect: return launch_split_form<kMassDefect>(e, partials, st, tr);
    case kMassDF: return launch_split_form<kMassDF>(e, partials, st, tr);
    default: return launch_split_form<kMassDefectDF>(e, partials, st, tr);
  }
}

// Enqueue one step on `st` (also used under stream capture).
int enqueue_step(gbf_ensemble* e, cudaStream_t st) {
  const bool mass = (e->out_flags & GBF_OUT_MASS) && e->d_mass_hist;
  double* partials = mass ? e->d_partials : nullptr;
  GbfTimer* tm = &e->timer;
  cudaEvent_t ev;
  if (e->precision != GBF_PREC_F64) {
    GBF_CUDA(cudaMemsetAsync(e->d_counter, 0, sizeof(unsigned), st));
    ev = gbf_timer_begin(tm, st);
    if (e->any_patch) k_ens_split_patch<<<e->n, 64, 0, st>>>(e->d_mem, 0, e->cur);  // timed with the step
    if (int s = launch_split_step(e, partials, st, {0, (int)e->tiles.size(), e->cur, e->d_counter, e->d_order}))
      return s;
    gbf_timer_end(tm, GBF_K_ENS_STEP, ev, st);
    ev = gbf_timer_begin(tm, st);
    if (kShapePairs[e->shape])
      k_ens_split_faces<<<(unsigned)e->bnd.size(), kThreads, 0, st>>>(e->d_mem, e->d_bnd, e->cur);
    else
      k_ens_split_boundary<<<(unsigned)e->bnd.size(), kThreads, 0, st>>>(e->d_mem, e->d_bnd, e->cur);
    gbf_timer_end(tm, GBF_K_ENS_BOUNDARY, ev, st);
  } else {
    ev = gbf_timer_begin(tm, st);
    k_ens_f64_props<<<(unsigned)e->props.size(), kThreads, 0, st>>>(e->d_mem, e->d_props, e->cur);
    gbf_timer_end(tm, GBF_K_ENS_PROPS, ev, st);
    ev = gbf_timer_begin(tm, st);
    k_ens_f64_flux_newton<<<(unsigned)e->flux.size(), kThreads, 0, st>>>(e->d_mem, e->d_flux, e->cur, partials,
                                                                         e->d_status);
    gbf_timer_end(tm, GBF_K_ENS_FLUX_NEWTON, ev, st);
    ev = gbf_timer_begin(tm, st);
    k_ens_f64_boundary<<<(unsigned)e->bnd.size(), kThreads, 0, st>>>(e->d_mem, e->d_bnd, e->cur);
    gbf_timer_end(tm, GBF_K_ENS_BOUNDARY, ev, st);
  }
  if (mass) {
    ev = gbf_timer_begin(tm, st);
    k_ens_mass_tail<<<e->n, 256, 0, st>>>(e->d_mem, e->d_partials, e->d_mass_hist, e->d_mass_count, e->n, e->mass_cap);
    k_ens_count<<<1, 1, 0, st>>>(e->d_mass_count);
    gbf_timer_end(tm, GBF_K_MASS_TAIL, ev, st);
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? GBF_OK : gbf_cuda_check(err, "gbf_ensemble step");
}

int capture_graph(gbf_ensemble* e, int parity) {
  const int saved = e->cur;
  e->cur = parity;
  cudaGraph_t g = nullptr;
  GBF_CUDA(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
  int s = enqueue_step(e, e->stream);
  cudaError_t r = cudaStreamEndCapture(e->stream, &g);
  e->cur = saved;
  if (s) return s;
  if (r != cudaSuccess) return gbf_cuda_check(r, "end capture");
  r = cudaGraphInstantiate(&e->graph[parity], g, 0);
  cudaGraphDestroy(g);
  return r == cudaSuccess ? GBF_OK : gbf_cuda_check(r, "graph instantiate");
}

int ens_step(gbf_ensemble* e, int nsteps, bool use_graph) {
  for (int q = 0; q < nsteps; q++) {
    if (use_graph && !e->timer.on) {
      if (!e->graph[e->cur])
        if (int s = capture_graph(e, e->cur)) return s;
      GBF_CUDA(cudaGraphLaunch(e->graph[e->cur], e->stream));
    } else {
      if (int s = enqueue_step(e, e->stream)) return s;
    }
    e->cur ^= 1;
    e->steps++;
  }
  return GBF_OK;
}

// One step of members [r0, r1) at buffer parity `cur` on `st`: their tiles
// (or chunks) and faces only, no phase-mass reduction.
int enqueue_group_step(gbf_ensemble* e, int r0, int r1, int cur, unsigned* counter, cudaStream_t st) {
  const auto &a = e->starts[r0], &b = e->starts[r1];
  if (e->precision != GBF_PREC_F64) {
    GBF_CUDA(cudaMemsetAsync(counter, 0, sizeof(unsigned), st));
    if (e->any_patch) k_ens_split_patch<<<r1 - r0, 64, 0, st>>>(e->d_mem, r0, cur);
    if (int s = launch_split_step(e, nullptr, st, {a.tiles, b.tiles - a.tiles, cur, counter, nullptr})) return s;
    if (kShapePairs[e->shape])
      k_ens_split_faces<<<(unsigned)(b.bnd - a.bnd), kThreads, 0, st>>>(e->d_mem, e->d_bnd + a.bnd, cur);
    else
      k_ens_split_boundary<<<(unsigned)(b.bnd - a.bnd), kThreads, 0, st>>>(e->d_mem, e->d_bnd + a.bnd, cur);
  } else {
    k_ens_f64_props<<<(unsigned)(b.props - a.props), kThreads, 0, st>>>(e->d_mem, e->d_props + a.props, cur);
    k_ens_f64_flux_newton<<<(unsigned)(b.flux - a.flux), kThreads, 0, st>>>(e->d_mem, e->d_flux + a.flux, cur,
                                                                           nullptr, e->d_status);
    k_ens_f64_boundary<<<(unsigned)(b.bnd - a.bnd), kThreads, 0, st>>>(e->d_mem, e->d_bnd + a.bnd, cur);
  }
  cudaError_t err = cudaGetLastError();
  return err == cudaSuccess ? GBF_OK : gbf_cuda_check(err, "gbf_ensemble group step");
}

// Member groups of the host-resident pipeline: contiguous ranges, at least
// kPipeCells cells each, at most kPipeGroups groups. The first and the last
// group take a quarter share of the cells and the others a full one: the
// first group's upload and the last group's download are the only copies
// that nothing overlaps, so small end groups shorten the pipeline's fill and
// drain.
constexpr long long kPipeCells = 4ll << 20;
constexpr int kPipeGroups = 16;
std::vector<int> pipe_groups(const gbf_ensemble* e) {
  const long long want = std::max(1ll, std::min<long long>({(long long)kPipeGroups, (long long)e->n,
                                                              e->pipe_groups > 0 ? e->pipe_groups : e->cells / kPipeCells}));
  // cumulative share of group g's end: (g + 1 - 0.75) / (want - 1.5) for g < want - 1 (want >= 3)
  auto end_share = [&](long long g) {
    if (want < 3) return (double)(g + 1) / (double)want;
    return ((double)g + 0.25) / ((double)want - 1.5);
  };
  std::vector<int> first = {0};
  long long acc = 0;
  for (int r = 0; r < e->n; r++) {
    acc += (long long)gbf_geo(e->models[r]).n;
    const long long g = (long long)first.size() - 1;  // the group member r belongs to
    if (r + 1 < e->n && g + 1 < want && (double)acc >= end_share(g) * (double)e->cells) first.push_back(r + 1);
  }
  first.push_back(e->n);
  return first;
}

int ensure_pipe(gbf_ensemble* e, int groups) {
  if (!e->s_in) {
    GBF_CUDA(cudaStreamCreateWithFlags(&e->s_in, cudaStreamNonBlocking));
    GBF_CUDA(cudaStreamCreateWithFlags(&e->s_out, cudaStreamNonBlocking));
    if (int s = ens_alloc(e, (void**)&e->d_gcounter, sizeof(unsigned) * kPipeGroups)) return s;
  }
  while ((int)e->ev.size() < 2 + 2 * groups) {
    cudaEvent_t v;
    GBF_CUDA(cudaEventCreateWithFlags(&v, cudaEventDisableTiming));
    e->ev.push_back(v);
  }
  return GBF_OK;
}

}  // namespace

extern "C" {

int gbf_ensemble_create(int n, const gbf_model* models, const gbf_cells* host_cells, int precision,
                        gbf_ensemble** out) {
  if (!out || n < 1 || !models) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_create");
  *out = nullptr;
  if (precision != GBF_PREC_F64 && precision != GBF_PREC_SPLIT && precision != GBF_PREC_SPLIT_DF &&
      precision != GBF_PREC_SPLIT_DEFECT)
    return gbf_fail(GBF_ERR_ARG, "precision");
  for (int r = 0; r < n; r++)
    if (int s = gbf_model_validate(&models[r], host_cells ? &host_cells[r] : nullptr, 0)) return s;
  gbf_ensemble* e = new gbf_ensemble();
  e->n = n;
  e->precision = precision;
  e->models.assign(models, models + n);
  e->h_mem.resize(n);
  int s = GBF_OK;
  if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking) != cudaSuccess) s = gbf_fail(GBF_ERR_CUDA, "stream");
  e->own_stream = true;
  const bool split = precision != GBF_PREC_F64;
  for (int r = 0; r < n && !s; r++) {
    const gbf_model& m = models[r];
    const size_t nc = gbf_geo(m).n;
    e->cells += (long long)nc;
    EnsMember& me = e->h_mem[r];
    memset(&me, 0, sizeof(me));
    me.off = (unsigned long long)(e->cells - (long long)nc);
    me.m = m;
    me.d = gbf_derive(m);
    me.C = gbf_split_consts(m);
    if (host_cells) {
      const gbf_cells& hc = host_cells[r];
      if (hc.media && !(s |= ens_alloc(e, (void**)&me.cells.media, nc * sizeof(int))))
        cudaMemcpy((void*)me.cells.media, hc.media, nc * sizeof(int), cudaMemcpyHostToDevice);
      if (hc.K && !(s |= ens_alloc(e, (void**)&me.cells.K, nc * sizeof(float))))
        cudaMemcpy((void*)me.cells.K, hc.K, nc * sizeof(float), cudaMemcpyHostToDevice);
      if (hc.phi && !(s |= ens_alloc(e, (void**)&me.cells.phi, nc * sizeof(float))))
        cudaMemcpy((void*)me.cells.phi, hc.phi, nc * sizeof(float), cudaMemcpyHostToDevice);
    }
    me.k1v = 0.0;
    if (split && !s && gbf_is_defect(gbf_mass_rep(precision)))
      s |= gbf_defect_k1(m, me.cells.phi, me.cells.media, &me.k1v, nullptr);
    if (split) {
      for (int b = 0; b < 2; b++) {
        s |= ens_alloc(e, (void**)&me.dPf[b], nc * sizeof(float));
        s |= ens_alloc(e, (void**)&me.Sf[b], nc * sizeof(float));
      }
      s |= ens_alloc(e, (void**)&me.M1, nc * gbf_mass_bytes(gbf_mass_rep(precision)));
      s |= ens_alloc(e, (void**)&me.M2, nc * gbf_mass_bytes(gbf_mass_rep(precision)));
      s |= ens_alloc(e, (void**)&me.rows, sizeof(GbfRowConst) * (size_t)m.ny);
      me.pc = gbf_patch_consts(m);
      if (me.pc.n > 0) {  // zeroed: entries outside the interior are never written (nor used)
        s |= ens_alloc(e, (void**)&me.patch, sizeof(float2) * (size_t)me.pc.n * me.pc.n);
        if (!s) s |= gbf_cuda_check(cudaMemset(me.patch, 0, sizeof(float2) * (size_t)me.pc.n * me.pc.n),
                                    "gbf_ensemble patch");
        e->any_patch = true;
      }
    } else {
      for (int b = 0; b < 2; b++) {
        s |= ens_alloc(e, (void**)&me.P[b], nc * sizeof(double));
        s |= ens_alloc(e, (void**)&me.S[b], nc * sizeof(double));
      }
      double** w[] = {&me.L1, &me.L2, &me.ro1, &me.ro2, &me.lnSe};
      for (double** p : w) s |= ens_alloc(e, (void**)p, nc * sizeof(double));
    }
  }
  if (!s) s |= ens_alloc(e, (void**)&e->d_counter, sizeof(unsigned));
  if (!s) s |= ens_alloc(e, (void**)&e->d_status, sizeof(unsigned));
  if (!s) s |= ens_alloc(e, (void**)&e->d_mass_count, sizeof(unsigned));
  if (!s) {
    cudaMemset(e->d_status, 0, sizeof(unsigned));
    cudaMemset(e->d_mass_count, 0, sizeof(unsigned));
    s = build_lists(e);
  }
  if (!s && e->precision != GBF_PREC_F64) {  // the members' row-constant tables, once
    k_ens_rows<<<e->n, 64>>>(e->d_mem);
    s = gbf_cuda_check(cudaDeviceSynchronize(), "gbf_ensemble_create rows");
  }
  if (s) {
    gbf_ensemble_destroy(e);
    return gbf_fail(s ? s : GBF_ERR_CUDA, "gbf_ensemble_create");
  }
  *out = e;
  return GBF_OK;
}

int gbf_ensemble_destroy(gbf_ensemble* e) {
  if (!e) return GBF_OK;
  if (e->stream) cudaStreamSynchronize(e->stream);
  if (e->s_out) cudaStreamSynchronize(e->s_out);
  drop_graphs(e);
  gbf_timer_free(&e->timer);
  for (cudaEvent_t v : e->ev) cudaEventDestroy(v);
  if (e->s_in) cudaStreamDestroy(e->s_in);
  if (e->s_out) cudaStreamDestroy(e->s_out);
  for (void* p : e->owned) cudaFree(p);
  if (e->own_stream && e->stream) cudaStreamDestroy(e->stream);
  delete e;
  return GBF_OK;
}

int gbf_ensemble_size(gbf_ensemble* e) { return e ? e->n : 0; }
long long gbf_ensemble_cells(gbf_ensemble* e) { return e ? e->cells : 0; }
long long gbf_ensemble_interior_cells(gbf_ensemble* e) {
  if (!e) return 0;
  long long s = 0;
  for (auto& m : e->models) s += (long long)(m.nx - 2) * (m.ny - 2) * (m.nz - 2);
  return s;
}

int gbf_ensemble_set_stream(gbf_ensemble* e, void* stream) {
  if (!e) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_set_stream");
  GBF_CUDA(cudaStreamSynchronize(e->stream));
  if (e->own_stream) cudaStreamDestroy(e->stream);
  e->stream = (cudaStream_t)stream;
  e->own_stream = false;
  drop_graphs(e);
  return GBF_OK;
}

int gbf_ensemble_set_outputs(gbf_ensemble* e, int flags, int mass_cap) {
  if (!e || mass_cap < 0 || (flags & ~(GBF_OUT_MASS | GBF_OUT_CFL)))
    return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_set_outputs");
  if ((flags & GBF_OUT_MASS) && mass_cap > e->mass_cap) {
    if (int s = ens_alloc(e, (void**)&e->d_mass_hist, 2 * sizeof(double) * (size_t)mass_cap * e->n)) return s;
    if (int s = ens_alloc(e, (void**)&e->d_cfl_hist, 2 * sizeof(float) * (size_t)mass_cap * e->n)) return s;
    e->mass_cap = mass_cap;
  }
  e->out_flags = flags;
  GBF_CUDA(cudaMemsetAsync(e->d_mass_count, 0, sizeof(unsigned), e->stream));
  if (e->d_cfl_hist)
    GBF_CUDA(cudaMemsetAsync(e->d_cfl_hist, 0, 2 * sizeof(float) * (size_t)e->mass_cap * e->n, e->stream));
  drop_graphs(e);
  return GBF_OK;
}

int gbf_ensemble_upload(gbf_ensemble* e, int r, const double* P1, const double* S2) {
  if (!e || r < 0 || r >= e->n || !P1 || !S2) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_upload");
  EnsMember& me = e->h_mem[r];
  const gbf_model& m = e->models[r];
  const size_t nc = gbf_geo(m).n, b = nc * sizeof(double);
  // all members share one buffer parity: write the member's current buffer
  const int c = e->cur;
  if (e->precision == GBF_PREC_F64) {
    GBF_CUDA(cudaMemcpyAsync(me.P[c], P1, b, cudaMemcpyDefault, e->stream));
    GBF_CUDA(cudaMemcpyAsync(me.S[c], S2, b, cudaMemcpyDefault, e->stream));
  } else {
    double* tmp = nullptr;
    GBF_CUDA(cudaMallocAsync((void**)&tmp, 2 * b, e->stream));
    GBF_CUDA(cudaMemcpyAsync(tmp, P1, b, cudaMemcpyDefault, e->stream));
    GBF_CUDA(cudaMemcpyAsync(tmp + nc, S2, b, cudaMemcpyDefault, e->stream));
    if (int s = gbf_split_init_state(m, me.rows, tmp, tmp + nc, me.dPf[c], me.Sf[c], me.M1, me.M2,
                                     gbf_mass_rep(e->precision), e->stream))
      return s;
    // the next-state buffer's faces are rewritten every step; start them equal
    GBF_CUDA(cudaMemcpyAsync(me.dPf[c ^ 1], me.dPf[c], nc * sizeof(float), cudaMemcpyDeviceToDevice, e->stream));
    GBF_CUDA(cudaMemcpyAsync(me.Sf[c ^ 1], me.Sf[c], nc * sizeof(float), cudaMemcpyDeviceToDevice, e->stream));
    GBF_CUDA(cudaFreeAsync(tmp, e->stream));
  }
  e->steps = 0;
  GBF_CUDA(cudaMemsetAsync(e->d_status, 0, sizeof(unsigned), e->stream));
  GBF_CUDA(cudaMemsetAsync(e->d_mass_count, 0, sizeof(unsigned), e->stream));
  if (e->d_cfl_hist)
    GBF_CUDA(cudaMemsetAsync(e->d_cfl_hist, 0, 2 * sizeof(float) * (size_t)e->mass_cap * e->n, e->stream));
  return GBF_OK;
}

// Whole-ensemble transfers through one staging buffer of 2 x cells doubles
// (allocated on first use): one copy each way for all members and one
// conversion kernel, instead of per-member copies.
static int ensure_stage(gbf_ensemble* e) {
  if (e->d_stage) return GBF_OK;
  return ens_alloc(e, (void**)&e->d_stage, 2 * sizeof(double) * (size_t)e->cells);
}

int gbf_ensemble_upload_all(gbf_ensemble* e, const double* P_all, const double* S_all) {
  if (!e || !P_all || !S_all) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_upload_all");
  // page-locked host arrays: the conversion kernel reads them in place
  const double* P = (const double*)gbf_mapped_host(P_all);
  const double* S = (const double*)gbf_mapped_host(S_all);
  if (!P || !S) {
    if (int s = ensure_stage(e)) return s;
    const size_t b = sizeof(double) * (size_t)e->cells;
    GBF_CUDA(cudaMemcpyAsync(e->d_stage, P_all, b, cudaMemcpyDefault, e->stream));
    GBF_CUDA(cudaMemcpyAsync(e->d_stage + e->cells, S_all, b, cudaMemcpyDefault, e->stream));
    P = e->d_stage;
    S = e->d_stage + e->cells;
  }
  k_ens_load<<<(unsigned)e->all.size(), kThreads, 0, e->stream>>>(e->d_mem, e->d_all, e->cur, P, S, e->precision);
  GBF_CUDA(cudaGetLastError());
  e->steps = 0;
  GBF_CUDA(cudaMemsetAsync(e->d_status, 0, sizeof(unsigned), e->stream));
  GBF_CUDA(cudaMemsetAsync(e->d_mass_count, 0, sizeof(unsigned), e->stream));
  if (e->d_cfl_hist)
    GBF_CUDA(cudaMemsetAsync(e->d_cfl_hist, 0, 2 * sizeof(float) * (size_t)e->mass_cap * e->n, e->stream));
  // the host arrays may be reused as soon as this returns
  GBF_CUDA(cudaStreamSynchronize(e->stream));
  return GBF_OK;
}

int gbf_ensemble_download_all(gbf_ensemble* e, double* P_all, double* S_all) {
  if (!e || !P_all || !S_all) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_download_all");
  // page-locked host arrays: the conversion kernel writes them in place
  double* P = (double*)gbf_mapped_host(P_all);
  double* S = (double*)gbf_mapped_host(S_all);
  if (P && S) {
    k_ens_store<<<(unsigned)e->all.size(), kThreads, 0, e->stream>>>(e->d_mem, e->d_all, e->cur, P, S, e->precision);
    GBF_CUDA(cudaGetLastError());
  } else {
    if (int s = ensure_stage(e)) return s;
    const size_t b = sizeof(double) * (size_t)e->cells;
    k_ens_store<<<(unsigned)e->all.size(), kThreads, 0, e->stream>>>(e->d_mem, e->d_all, e->cur, e->d_stage,
                                                                     e->d_stage + e->cells, e->precision);
    GBF_CUDA(cudaGetLastError());
    GBF_CUDA(cudaMemcpyAsync(P_all, e->d_stage, b, cudaMemcpyDefault, e->stream));
    GBF_CUDA(cudaMemcpyAsync(S_all, e->d_stage + e->cells, b, cudaMemcpyDefault, e->stream));
  }
  GBF_CUDA(cudaStreamSynchronize(e->stream));
  return GBF_OK;
}

namespace {
int ens_advance_host(gbf_ensemble* e, const double* P_in, const double* S_in, int nsteps, double* P_out,
                     double* S_out) {
  if (int s = ensure_stage(e)) return s;
  const std::vector<int> first = pipe_groups(e);
  const int G = (int)first.size() - 1;
  if (int s = ensure_pipe(e, G)) return s;
  double *stP = e->d_stage, *stS = e->d_stage + e->cells;
  cudaStream_t cs = e->stream;
  // everything earlier on the ensemble's stream comes first
  GBF_CUDA(cudaMemsetAsync(e->d_status, 0, sizeof(unsigned), cs));
  GBF_CUDA(cudaEventRecord(e->ev[0], cs));
  GBF_CUDA(cudaStreamWaitEvent(e->s_in, e->ev[0], 0));
  GBF_CUDA(cudaStreamWaitEvent(e->s_out, e->ev[0], 0));
  auto span = [&](int g, size_t& off, size_t& bytes) {
    off = (size_t)e->h_mem[first[g]].off;
    const size_t end = first[g + 1] < e->n ? (size_t)e->h_mem[first[g + 1]].off : (size_t)e->cells;
    bytes = (end - off) * sizeof(double);
  };
  // host -> device copies of every group, in order, on the input stream
  for (int g = 0; g < G; g++) {
    size_t off, bytes;
    span(g, off, bytes);
    GBF_CUDA(cudaMemcpyAsync(stP + off, P_in + off, bytes, cudaMemcpyDefault, e->s_in));
    GBF_CUDA(cudaMemcpyAsync(stS + off, S_in + off, bytes, cudaMemcpyDefault, e->s_in));
    GBF_CUDA(cudaEventRecord(e->ev[2 + 2 * g], e->s_in));
  }
  // per group: load, nsteps steps, store (compute stream); device -> host copy (output stream)
  const int c0 = e->cur;
  for (int g = 0; g < G; g++) {
    const auto &a = e->starts[first[g]], &b = e->starts[first[g + 1]];
    GBF_CUDA(cudaStreamWaitEvent(cs, e->ev[2 + 2 * g], 0));
    k_ens_load<<<(unsigned)(b.all - a.all), kThreads, 0, cs>>>(e->d_mem, e->d_all + a.all, c0, stP, stS, e->precision);
    for (int q = 0; q < nsteps; q++)
      if (int s = enqueue_group_step(e, first[g], first[g + 1], c0 ^ (q & 1), e->d_gcounter + g, cs)) return s;
    k_ens_store<<<(unsigned)(b.all - a.all), kThreads, 0, cs>>>(e->d_mem, e->d_all + a.all, c0 ^ (nsteps & 1), stP,
                                                                 stS, e->precision);
    GBF_CUDA(cudaGetLastError());
    GBF_CUDA(cudaEventRecord(e->ev[3 + 2 * g], cs));
    GBF_CUDA(cudaStreamWaitEvent(e->s_out, e->ev[3 + 2 * g], 0));
    size_t off, bytes;
    span(g, off, bytes);
    GBF_CUDA(cudaMemcpyAsync(P_out + off, stP + off, bytes, cudaMemcpyDefault, e->s_out));
    GBF_CUDA(cudaMemcpyAsync(S_out + off, stS + off, bytes, cudaMemcpyDefault, e->s_out));
  }
  GBF_CUDA(cudaEventRecord(e->ev[1], e->s_out));
  GBF_CUDA(cudaStreamWaitEvent(cs, e->ev[1], 0));
  e->cur = c0 ^ (nsteps & 1);
  e->steps = nsteps;
  GBF_CUDA(cudaMemsetAsync(e->d_mass_count, 0, sizeof(unsigned), cs));
  if (e->d_cfl_hist)
    GBF_CUDA(cudaMemsetAsync(e->d_cfl_hist, 0, 2 * sizeof(float) * (size_t)e->mass_cap * e->n, cs));
  GBF_CUDA(cudaStreamSynchronize(cs));
  return GBF_OK;
}
}  // namespace

int gbf_ensemble_advance_host(gbf_ensemble* e, const double* P_in, const double* S_in, int nsteps, double* P_out,
                              double* S_out) {
  if (!e || !P_in || !S_in || !P_out || !S_out || nsteps < 0)
    return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_advance_host");
  const int s = ens_advance_host(e, P_in, S_in, nsteps, P_out, S_out);
  if (s) {  // an error part-way: no copy may still read or write the caller's arrays after the return
    if (e->s_in) cudaStreamSynchronize(e->s_in);
    if (e->s_out) cudaStreamSynchronize(e->s_out);
    cudaStreamSynchronize(e->stream);
  }
  return s;
}

int gbf_ensemble_set_pipeline_groups(gbf_ensemble* e, int groups) {
  if (!e || groups < 0) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_set_pipeline_groups");
  e->pipe_groups = groups;
  return GBF_OK;
}

int gbf_ensemble_step(gbf_ensemble* e, int nsteps) {
  if (!e || nsteps < 0) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_step");
  return ens_step(e, nsteps, true);
}

int gbf_ensemble_sync(gbf_ensemble* e) {
  if (!e) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_sync");
  GBF_CUDA(cudaStreamSynchronize(e->stream));
  return GBF_OK;
}

int gbf_ensemble_status(gbf_ensemble* e) {
  if (!e) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_status");
  unsigned h = 0;
  GBF_CUDA(cudaMemcpyAsync(&h, e->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, e->stream));
  GBF_CUDA(cudaStreamSynchronize(e->stream));
  if (h & GBF_DEV_TIMEOUT) return gbf_fail(GBF_ERR_TIMEOUT, "device wait timed out");
  if (h & GBF_DEV_NONFINITE) return gbf_fail(GBF_ERR_NONFINITE, "non-finite P or S");
  return GBF_OK;
}

int gbf_ensemble_download(gbf_ensemble* e, int r, int field, double* host) {
  if (!e || r < 0 || r >= e->n || !host || (field != GBF_FIELD_P1 && field != GBF_FIELD_S2))
    return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_download");
  const EnsMember& me = e->h_mem[r];
  const gbf_model& m = e->models[r];
  const size_t nc = gbf_geo(m).n, b = nc * sizeof(double);
  if (e->precision == GBF_PREC_F64) {
    GBF_CUDA(cudaMemcpyAsync(host, field == GBF_FIELD_P1 ? me.P[e->cur] : me.S[e->cur], b, cudaMemcpyDefault, e->stream));
  } else {
    double* tmp = nullptr;
    GBF_CUDA(cudaMallocAsync((void**)&tmp, b, e->stream));
    if (int s = gbf_split_state_to_f64(m, me.rows, me.dPf[e->cur], me.Sf[e->cur], field == GBF_FIELD_P1 ? tmp : nullptr,
                                       field == GBF_FIELD_S2 ? tmp : nullptr, e->stream))
      return s;
    GBF_CUDA(cudaMemcpyAsync(host, tmp, b, cudaMemcpyDefault, e->stream));
    GBF_CUDA(cudaFreeAsync(tmp, e->stream));
  }
  GBF_CUDA(cudaStreamSynchronize(e->stream));
  return GBF_OK;
}

int gbf_ensemble_mass_history(gbf_ensemble* e, double* host, int max_steps, int* nsteps_out) {
  if (!e || !host || max_steps < 0) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_mass_history");
  unsigned cnt = 0;
  GBF_CUDA(cudaMemcpyAsync(&cnt, e->d_mass_count, sizeof(unsigned), cudaMemcpyDeviceToHost, e->stream));
  GBF_CUDA(cudaStreamSynchronize(e->stream));
  int n = (int)std::min<unsigned>(cnt, (unsigned)std::min(max_steps, e->mass_cap));
  if (n > 0)
    GBF_CUDA(cudaMemcpy(host, e->d_mass_hist, 2 * sizeof(double) * (size_t)n * e->n, cudaMemcpyDeviceToHost));
  if (nsteps_out) *nsteps_out = n;
  return GBF_OK;
}

int gbf_ensemble_cfl_history(gbf_ensemble* e, float* host, int max_steps, int* nsteps_out) {
  if (!e || !host || max_steps < 0) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_cfl_history");
  unsigned cnt = 0;
  GBF_CUDA(cudaMemcpyAsync(&cnt, e->d_mass_count, sizeof(unsigned), cudaMemcpyDeviceToHost, e->stream));
  GBF_CUDA(cudaStreamSynchronize(e->stream));
  int n = (int)std::min<unsigned>(cnt, (unsigned)std::min(max_steps, e->mass_cap));
  if (n > 0 && e->d_cfl_hist)
    GBF_CUDA(cudaMemcpy(host, e->d_cfl_hist, 2 * sizeof(float) * (size_t)n * e->n, cudaMemcpyDeviceToHost));
  if (nsteps_out) *nsteps_out = n;
  return GBF_OK;
}

int gbf_ensemble_set_timing(gbf_ensemble* e, int on) {
  if (!e) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_set_timing");
  e->timer.on = on != 0;
  return GBF_OK;
}

int gbf_ensemble_kernel_times(gbf_ensemble* e, double* ms, int* launches, int nkinds) {
  if (!e || !ms || !launches) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_kernel_times");
  return gbf_timer_collect(&e->timer, ms, launches, nkinds);
}

int gbf_ensemble_launches_per_step(gbf_ensemble* e) {
  if (!e) return 0;
  const int mass = (e->out_flags & GBF_OUT_MASS) ? 2 : 0;
  return (e->precision == GBF_PREC_F64 ? 3 : 2 + (e->any_patch ? 1 : 0)) + mass;
}

int gbf_ensemble_set_tuning(gbf_ensemble* e, int shape, int edge, int kchunk) {
  if (!e || shape < -1 || shape >= kShapes || kchunk < 0) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_set_tuning");
  GBF_CUDA(cudaStreamSynchronize(e->stream));
  const int prev = e->shape;
  if (shape >= 0) e->shape = shape;
  if (edge > 0) e->kchunk_by_edge[edge] = kchunk;
  int s = build_lists(e);
  if (s && e->shape != prev) {  // e.g. the x-pair tile without TMA: keep the previous shape
    e->shape = prev;
    build_lists(e);
  }
  return s;
}

int gbf_ensemble_uses_tma(gbf_ensemble* e) { return e && e->d_maps ? 1 : 0; }

int gbf_ensemble_get_tuning(gbf_ensemble* e, int* shape, int* edges, int* kchunks, int max_entries) {
  if (!e || !shape) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_get_tuning");
  *shape = e->shape;
  int q = 0;
  for (auto& kv : e->kchunk_by_edge) {
    if (q >= max_entries) break;
    if (edges) edges[q] = kv.first;
    if (kchunks) kchunks[q] = kv.second;
    q++;
  }
  return q;
}

const char* gbf_ensemble_shape_name(int shape) {
  static const char* names[kShapes] = {"32x8", "64x4", "32x4", "64x8 pairs", "32x16 pairs", "32x16 + 48x10 pairs"};
  return (shape >= 0 && shape < kShapes) ? names[shape] : "";
}

// Pick the tile shape, then the fusion depth of every member edge, each by
// timing `trial_steps` steps per candidate (CUDA events on the ensemble's
// stream). Advances the state: upload the initial state after tuning.
int gbf_ensemble_autotune(gbf_ensemble* e, int trial_steps) {
  if (!e || trial_steps < 1) return gbf_fail(GBF_ERR_ARG, "gbf_ensemble_autotune");
  if (e->precision == GBF_PREC_F64) return GBF_OK;  // FP64 kernels: chunked, nothing to tune
  const bool timing = e->timer.on;
  e->timer.on = false;
  cudaEvent_t a, b;
  cudaEventCreate(&a);
  cudaEventCreate(&b);
  auto trial = [&](float& ms) -> int {
    if (int s = ens_step(e, 1, false)) return s;  // warm
    cudaEventRecord(a, e->stream);
    if (int s = ens_step(e, trial_steps, false)) return s;
    cudaEventRecord(b, e->stream);
    GBF_CUDA(cudaEventSynchronize(b));
    cudaEventElapsedTime(&ms, a, b);
    return GBF_OK;
  };
  int st = GBF_OK;
  // 1. tile shape, with the default fusion depth
  float best = 1e30f;
  int best_shape = e->shape;
  for (int sh = 0; sh < kShapes && !st; sh++) {
    if (kShapePairs[sh] && !tma_possible(e, kShapeTX[sh])) continue;
    e->shape = sh;
    if ((st = build_lists(e))) break;
    float ms = 0;
    if ((st = trial(ms))) break;
    if (ms < best) { best = ms; best_shape = sh; }
  }
  e->shape = best_shape;
  // 2. fusion depth per member edge (k planes per tile pass)
  std::vector<int> edges;
  for (auto& m : e->models)
    if (std::find(edges.begin(), edges.end(), m.nx) == edges.end()) edges.push_back(m.nx);
  const int cands[] = {16, 32, 64, 0};
  for (int edge : edges) {
    if (st) break;
    int best_kc = 0;
    float bt = 1e30f;
    for (int kc : cands) {
      e->kchunk_by_edge[edge] = kc;
      if ((st = build_lists(e))) break;
      float ms = 0;
      if ((st = trial(ms))) break;
      if (ms < bt) { bt = ms; best_kc = kc; }
    }
    e->kchunk_by_edge[edge] = best_kc;
  }
  if (!st) st = build_lists(e);
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  e->timer.on = timing;
  return st;
}

}  // extern "C"
