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

// Row count of the interior box of an 8-byte field (M1, M2): TX + 2 columns
// from x = i0 - 1 (inner extent a multiple of 16 bytes for even TX).
__host__ __device__ constexpr int gbf_tma_rows_x8(int TX) { return TX + 2; }

bool gbf_tma_enabled();
bool gbf_tma_eligible(int nx, int TX);
// Halo-plane box {gbf_tma_box_x(TX), TY + 2, 1} of an FP32 field.
int gbf_tma_encode_plane(void* map_out, const float* base, int nx, int ny, int nz, int TX, int TY);
// Interior-rows box of a field of 4-byte (FP32) or 8-byte elements:
// {gbf_tma_box_x(TX) or gbf_tma_rows_x8(TX), TY, 1}.
int gbf_tma_encode_rows(void* map_out, const void* base, int elem_bytes, int nx, int ny, int nz, int TX, int TY);

// Any {bx, by, 1} box of a field of 4- or 8-byte elements.
int gbf_tma_encode_box(void* map_out, const void* base, int elem_bytes, int nx, int ny, int nz, int bx, int by);

// The plane maps of one grid: halo planes of dP and S (both state buffers)
// and K; interior rows of the phase masses M1, M2 (8 bytes a cell) and phi.
struct GbfTmaSet {
  GbfTensorMap dP[2], S[2], K, M1, M2, phi;
};
