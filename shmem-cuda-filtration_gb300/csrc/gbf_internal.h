// gbf_internal.h — shared host/device helpers of libgbflow (not installed).
#pragma once

#include <cuda_runtime.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>

#include "../../include/gbflow.h"

#define GBF_HD __host__ __device__ __forceinline__

// ------------------------------------------------------------------ status
// Sticky status shared by all entry points (single host thread, like the
// reference). Returns `s` so callers can `return gbf_fail(...)`.
int gbf_fail(int s, const char* where);
int gbf_cuda_check(cudaError_t e, const char* where);
// Device address of a page-locked host array (cudaHostAlloc, cudaHostRegister)
// that kernels may access in place; NULL for pageable memory or when direct
// host access is switched off (gbf_set_host_direct).
const void* gbf_mapped_host(const void* p);
#define GBF_CUDA(call) do { cudaError_t e_ = (call); if (e_ != cudaSuccess) return gbf_cuda_check(e_, #call); } while (0)

// ---------------------------------------------------------------- geometry
struct GbfGeo {
  int nx, ny, nz;
  size_t pl;  // nx * ny
  size_t n;   // nx * ny * nz
};

GBF_HD GbfGeo gbf_geo(const gbf_model& m) {
  GbfGeo g;
  g.nx = m.nx; g.ny = m.ny; g.nz = m.nz;
  g.pl = (size_t)m.nx * (size_t)m.ny;
  g.n = g.pl * (size_t)m.nz;
  return g;
}
GBF_HD size_t gbf_idx(const GbfGeo& g, int i, int j, int k) { return (size_t)i + (size_t)j * g.nx + (size_t)k * g.pl; }
GBF_HD bool gbf_is_boundary(const GbfGeo& g, int i, int j, int k) {
  return i == 0 || i == g.nx - 1 || j == 0 || j == g.ny - 1 || k == 0 || k == g.nz - 1;
}

// Boundary cells enumerated compactly (grid dims >= 3):
//   [0, 2*nx*ny)                      faces k = 0 and k = nz-1 (all i, j)
//   [.., + 2*nx*(nz-2))               faces j = 0 and j = ny-1 (k interior)
//   [.., + 2*(ny-2)*(nz-2))           faces i = 0 and i = nx-1 (j, k interior)
GBF_HD size_t gbf_boundary_count(const GbfGeo& g) {
  return 2 * g.pl + 2 * (size_t)g.nx * (g.nz - 2) + 2 * (size_t)(g.ny - 2) * (g.nz - 2);
}
// The first two groups only: every boundary cell but the x faces with j, k
// interior (which the x-pair split tile writes itself).
GBF_HD size_t gbf_boundary_count_no_xfaces(const GbfGeo& g) { return 2 * g.pl + 2 * (size_t)g.nx * (g.nz - 2); }
// The same cells as rows of nx cells at (j, k), "face rows":
//   r in [0, 2 ny)                  k = 0 (r < ny) or nz - 1, j = r mod ny
//   r in [2 ny, 2 ny + 2 (nz - 2))  j = 0 or ny - 1, k = 1 + (r - 2 ny) mod (nz - 2)
GBF_HD int gbf_face_rows(const GbfGeo& g) { return 2 * g.ny + 2 * (g.nz - 2); }
GBF_HD void gbf_face_row(const GbfGeo& g, int r, int& j, int& k) {
  if (r < 2 * g.ny) {
    k = r < g.ny ? 0 : g.nz - 1;
    j = r < g.ny ? r : r - g.ny;
    return;
  }
  r -= 2 * g.ny;
  const int nk = g.nz - 2;
  j = r < nk ? 0 : g.ny - 1;
  k = 1 + (r < nk ? r : r - nk);
}
// (i, j, k) of boundary cell `id` in the order above. 32-bit arithmetic:
// grids hold fewer than 2^31 cells (checked on the host), and 64-bit
// division is emulated on the GPU.
GBF_HD void gbf_boundary_cell(const GbfGeo& g, size_t id_, int& i, int& j, int& k) {
  unsigned id = (unsigned)id_;
  const unsigned nx = (unsigned)g.nx, pl = (unsigned)g.pl;
  const unsigned a = 2u * pl;
  if (id < a) {
    k = id < pl ? 0 : g.nz - 1;
    const unsigned r = id < pl ? id : id - pl;
    j = (int)(r / nx);
    i = (int)(r - (unsigned)j * nx);
    return;
  }
  id -= a;
  const unsigned face = nx * (unsigned)(g.nz - 2);
  if (id < 2u * face) {
    j = id < face ? 0 : g.ny - 1;
    const unsigned r = id < face ? id : id - face;
    const unsigned q = r / nx;
    k = 1 + (int)q;
    i = (int)(r - q * nx);
    return;
  }
  id -= 2u * face;
  const unsigned ry = (unsigned)(g.ny - 2), face_x = ry * (unsigned)(g.nz - 2);
  i = id < face_x ? 0 : g.nx - 1;
  const unsigned r = id < face_x ? id : id - face_x;
  const unsigned q = r / ry;
  k = 1 + (int)q;
  j = 1 + (int)(r - q * ry);
}

// Top-centre Dirichlet patch of the reference, |I - NX/2| <= source (cpu.cpp:346).
GBF_HD bool gbf_in_dirichlet_patch(const gbf_model& m, int i, int k) {
  return (i >= m.nx / 2 - m.source) && (i <= m.nx / 2 + m.source) &&
         (k >= m.nz / 2 - m.source) && (k <= m.nz / 2 + m.source);
}
// Rate-injection patch: n x n cells centred like the reference patch.
GBF_HD bool gbf_in_rate_patch(const gbf_model& m, int i, int k) {
  int n = m.rate_cells, i0 = m.nx / 2 - n / 2, k0 = m.nz / 2 - n / 2;
  return (i >= i0) && (i < i0 + n) && (k >= k0) && (k < k0 + n);
}
// Initial hydrostatic profile (main.cpp:114); also the Dirichlet side value.
GBF_HD double gbf_p_hydrostatic(const gbf_model& m, int j) { return m.P_atm + j * m.ro01 * m.g * (m.h2); }

// --------------------------------------------------- boundary sweep values
// The reference applies Border_S2 then Border_P1 to every cell in one
// i -> j -> k sweep, in place (cpu.cpp:44-54, 323-403). A boundary cell
// therefore sees the NEW value of a neighbour that comes earlier in the sweep
// and the OLD value of one that comes later. The functions below return the
// value the sweep leaves at boundary cell (i, j, k) without running a sweep:
// they follow the chain of "copy from an earlier cell" rules (at most three
// hops) and read
//   cur[c]  for interior cells (their post-Newton value), and
//   old[c]  for boundary cells that come later in the sweep (untouched yet).
// Eager (in-place) kernels pass the same array as cur and old; the ping-pong
// kernels pass the new and the previous buffer.
template <class T>
GBF_HD T gbf_later(const GbfGeo& g, const T* cur, const T* old, int i, int j, int k) {
  size_t c = gbf_idx(g, i, j, k);
  return gbf_is_boundary(g, i, j, k) ? old[c] : cur[c];
}

template <class T>
GBF_HD T gbf_sweep_S(const gbf_model& m, const GbfGeo& g, const T* cur, const T* old, int i, int j, int k) {
  for (int hop = 0; hop < 6; ++hop) {
    if (i == 0) return gbf_later(g, cur, old, 1, j, k);
    if (i == g.nx - 1) { i = g.nx - 2; if (!gbf_is_boundary(g, i, j, k)) return cur[gbf_idx(g, i, j, k)]; continue; }
    if (j == g.ny - 1) { j = g.ny - 2; if (!gbf_is_boundary(g, i, j, k)) return cur[gbf_idx(g, i, j, k)]; continue; }
    if (j == 0) {
      // Dirichlet value first, then the k rules still apply (no return, cpu.cpp:343-351)
      if (k == 0) return gbf_later(g, cur, old, i, 0, 1);
      if (k == g.nz - 1) { k = g.nz - 2; continue; }  // (i, 0, nz-2): earlier, a j == 0 cell
      bool patch = (m.source_mode == GBF_SOURCE_DIRICHLET_PATCH) && gbf_in_dirichlet_patch(m, i, k);
      return patch ? (T)m.S2_gr : (T)0;
    }
    if (k == 0) return gbf_later(g, cur, old, i, j, 1);
    if (k == g.nz - 1) { k = g.nz - 2; if (!gbf_is_boundary(g, i, j, k)) return cur[gbf_idx(g, i, j, k)]; continue; }
    return cur[gbf_idx(g, i, j, k)];
  }
  return (T)NAN;
}

// `ro1_top(i)` is the start-of-step water density at (i, 1, 0) that the
// bottom rule reads for every k (cpu.cpp:382).
template <class T, class Ro1>
GBF_HD T gbf_sweep_P(const gbf_model& m, const GbfGeo& g, const T* cur, const T* old, int i, int j, int k,
                     Ro1 ro1_top) {
  bool has_add = false;
  T add = 0, base = (T)NAN;
  for (int hop = 0; hop < 6; ++hop) {
    if (m.bc_mode == GBF_BC_HYDROSTATIC_SIDES && (i == 0 || i == g.nx - 1 || k == 0 || k == g.nz - 1)) {
      base = (T)gbf_p_hydrostatic(m, j);
      break;
    }
    if (i == 0) { base = gbf_later(g, cur, old, 1, j, k); break; }
    if (i == g.nx - 1) {
      i = g.nx - 2;
      if (!gbf_is_boundary(g, i, j, k)) { base = cur[gbf_idx(g, i, j, k)]; break; }
      continue;
    }
    if (j == g.ny - 1) {
      add = ro1_top(i) * (T)m.g * (T)(m.h2);
      has_add = true;
      j = g.ny - 2;
      if (!gbf_is_boundary(g, i, j, k)) { base = cur[gbf_idx(g, i, j, k)]; break; }
      continue;
    }
    if (j == 0) { base = (T)m.P_atm; break; }
    if (k == 0) { base = gbf_later(g, cur, old, i, j, 1); break; }
    if (k == g.nz - 1) {
      k = g.nz - 2;
      if (!gbf_is_boundary(g, i, j, k)) { base = cur[gbf_idx(g, i, j, k)]; break; }
      continue;
    }
    base = cur[gbf_idx(g, i, j, k)];
    break;
  }
  return has_add ? base + add : base;
}

// ------------------------------------------------------- kernel timing
// Optional CUDA-event spans around each kernel launch, on the launching
// stream (bench accounting of the dominant kernel). Kinds index gbf_kernel_name().
enum { GBF_K_PROPS = 0, GBF_K_FLUX_NEWTON, GBF_K_BOUNDARY, GBF_K_MASS_TAIL, GBF_K_SPLIT_STEP, GBF_K_SPLIT_BOUNDARY,
       GBF_K_ENS_STEP, GBF_K_ENS_BOUNDARY, GBF_K_ENS_PROPS, GBF_K_ENS_FLUX_NEWTON, GBF_K_COUNT };

struct GbfTimer {
  bool on = false;
  struct Rec { int kind; cudaEvent_t a, b; };
  cudaEvent_t* pool = nullptr;
  size_t cap = 0, used = 0;
  Rec* recs = nullptr;
  size_t nrec = 0, rcap = 0;
  cudaEvent_t last = nullptr;  // end of the previous span on this stream
};
// Record the start of a span (returns its start event) and the end of it.
cudaEvent_t gbf_timer_begin(GbfTimer* t, cudaStream_t st);
void gbf_timer_end(GbfTimer* t, int kind, cudaEvent_t start, cudaStream_t st);
// Sum spans per kind (synchronises on the events); resets the timer.
int gbf_timer_collect(GbfTimer* t, double* ms, int* launches, int nkinds);
void gbf_timer_free(GbfTimer* t);

// ---------------------------------------------------------- launch helpers
int gbf_num_sms();
inline unsigned gbf_grid_for(size_t n, int threads, int per_sm = 8) {
  size_t want = (n + threads - 1) / threads;
  size_t cap = (size_t)gbf_num_sms() * per_sm;
  return (unsigned)(want < cap ? (want > 0 ? want : 1) : cap);
}
