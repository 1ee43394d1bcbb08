// gbf_tma.cpp — tensor maps of the split kernels' TMA plane loads.
//
// One map per FP32 field (dP, S of both ping-pong buffers, K) of a grid:
// a 3-D tensor {nx, ny, nz} and a box {TX + 4, TY + 2, 1}, i.e. one x-y
// plane of a tile with its 1-cell halo (the x extent rounded up so that the
// box's inner extent is a multiple of 16 bytes). The driver function is
// reached through the runtime's entry-point query, so libgbflow does not
// link libcuda directly.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <mutex>

#include "gbf_internal.h"
#include "gbf_tma.h"

namespace {
std::mutex g_mu;
PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;
std::atomic<int> g_tma_on{1};

PFN_cuTensorMapEncodeTiled_v12000 encoder() {
  std::lock_guard<std::mutex> lk(g_mu);
  if (!g_encode) {
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      g_encode = (PFN_cuTensorMapEncodeTiled_v12000)fn;
  }
  return g_encode;
}
}  // namespace

bool gbf_tma_enabled() { return g_tma_on.load() != 0; }

// Whether a grid can use the TMA plane loads: rows of whole 16-byte units
// (nx % 4 == 0) and a tile whose first halo column is 16-byte aligned
// (TX % 4 == 0; tiles start at x = tile * TX).
bool gbf_tma_eligible(int nx, int TX) { return gbf_tma_enabled() && nx % 4 == 0 && TX % 4 == 0 && encoder() != nullptr; }

namespace {
// A 3-D map {nx, ny, nz} of `eb`-byte elements with a {bx, by, 1} box.
int encode(void* map_out, const void* base, int eb, int nx, int ny, int nz, int bx, int by) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = encoder();
  if (!enc) return gbf_fail(GBF_ERR_CUDA, "cuTensorMapEncodeTiled unavailable");
  if (!base || ((uintptr_t)base & 15) != 0 || ((size_t)nx * eb) % 16 != 0 || (eb != 4 && eb != 8))
    return gbf_fail(GBF_ERR_ARG, "TMA map: alignment");
  if (bx > 256 || by > 256 || ((size_t)bx * eb) % 16 != 0) return gbf_fail(GBF_ERR_ARG, "TMA map: box");
  const cuuint64_t dims[3] = {(cuuint64_t)nx, (cuuint64_t)ny, (cuuint64_t)nz};
  const cuuint64_t strides[2] = {(cuuint64_t)nx * eb, (cuuint64_t)nx * ny * eb};  // bytes, dims 1 and 2
  const cuuint32_t box[3] = {(cuuint32_t)bx, (cuuint32_t)by, 1};
  const cuuint32_t elem[3] = {1, 1, 1};
  CUtensorMap m;
  CUresult r = enc(&m, eb == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, (void*)base,
                   dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) return gbf_fail(GBF_ERR_CUDA, "cuTensorMapEncodeTiled");
  memcpy(map_out, &m, sizeof(m));
  return GBF_OK;
}
}  // namespace

int gbf_tma_encode_plane(void* map_out, const float* base, int nx, int ny, int nz, int TX, int TY) {
  if (TX % 4 != 0) return gbf_fail(GBF_ERR_ARG, "TMA plane map: tile width");
  return encode(map_out, base, 4, nx, ny, nz, gbf_tma_box_x(TX), TY + 2);
}

int gbf_tma_encode_rows(void* map_out, const void* base, int elem_bytes, int nx, int ny, int nz, int TX, int TY) {
  if (TX % 4 != 0) return gbf_fail(GBF_ERR_ARG, "TMA rows map: tile width");
  return encode(map_out, base, elem_bytes, nx, ny, nz, elem_bytes == 8 ? gbf_tma_rows_x8(TX) : gbf_tma_box_x(TX), TY);
}

int gbf_tma_encode_box(void* map_out, const void* base, int elem_bytes, int nx, int ny, int nz, int bx, int by) {
  return encode(map_out, base, elem_bytes, nx, ny, nz, bx, by);
}

extern "C" int gbf_set_tma(int on) {
  if (on < 0) return g_tma_on.load();
  return g_tma_on.exchange(on ? 1 : 0);
}
