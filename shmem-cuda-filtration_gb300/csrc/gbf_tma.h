// gbf_tma.h — host side of the TMA plane loads (gbf_tma.cpp).
#pragma once

#include <cuda_runtime.h>

// 128-byte tensor map (CUtensorMap) storage, 64-byte aligned as the TMA unit requires.
struct alignas(64) GbfTensorMap {
  unsigned char bytes[128];
};

// Box width of a tile of TX columns: TX + 2 halo columns rounded up to 4
// floats (16 bytes).
__host__ __device__ constexpr int gbf_tma_box_x(int TX) { return ((TX + 2 + 3) / 4) * 4; }

bool gbf_tma_enabled();
bool gbf_tma_eligible(int nx, int TX);
int gbf_tma_encode_plane(void* map_out, const float* base, int nx, int ny, int nz, int TX, int TY);

// The five plane maps of one grid: dP and S of both state buffers, and K.
struct GbfTmaSet {
  GbfTensorMap dP[2], S[2], K;
};
