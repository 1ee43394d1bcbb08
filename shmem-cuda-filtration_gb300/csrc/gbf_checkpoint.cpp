// gbf_checkpoint.cpp — the reference's checkpoint file, host side.
//
// Layout of save/save.dat for one domain (main.cpp:485-538 save, 541-572
// restore; one record per rank, a single record here):
//   int    step
//   double P1[n], S2[n], x[n], y[n], z[n], roS1_old[n], roS2_old[n]
//   int    media[n]
// with n = nx*ny*nz, cell index i + j*nx + k*nx*ny, native byte order, no
// padding. x, y, z are the cell coordinates i*h1, j*h2, k*h3 that
// initial_data writes (main.cpp:115-117); the reader checks them against the
// model so that a file of another grid is refused.
#include <stdio.h>
#include <string.h>

#include <vector>

#include "gbf_internal.h"

namespace {

size_t cells_of(const gbf_model* m) { return (size_t)m->nx * m->ny * m->nz; }

// Coordinate arrays of main.cpp:115-117 for a single domain (I = i).
void coordinates(const gbf_model* m, int axis, std::vector<double>& out) {
  const size_t n = cells_of(m);
  out.resize(n);
  for (int k = 0; k < m->nz; k++)
    for (int j = 0; j < m->ny; j++)
      for (int i = 0; i < m->nx; i++) {
        const size_t c = (size_t)i + (size_t)j * m->nx + (size_t)k * m->nx * m->ny;
        out[c] = axis == 0 ? i * (m->h1) : axis == 1 ? j * (m->h2) : k * (m->h3);
      }
}

struct File {
  FILE* f = nullptr;
  ~File() {
    if (f) fclose(f);
  }
};

}  // namespace

extern "C" {

size_t gbf_checkpoint_bytes(const gbf_model* m) {
  if (!m || m->nx < 1 || m->ny < 1 || m->nz < 1) return 0;
  const size_t n = cells_of(m);
  return sizeof(int) + 7 * n * sizeof(double) + n * sizeof(int);
}

int gbf_checkpoint_write(const char* path, const gbf_model* m, int step, const double* P1, const double* S2,
                         const double* roS1_old, const double* roS2_old, const int* media) {
  if (!path || !m || !P1 || !S2 || gbf_checkpoint_bytes(m) == 0) return gbf_fail(GBF_ERR_ARG, "gbf_checkpoint_write");
  const size_t n = cells_of(m);
  std::vector<double> zeros, xyz;
  File out;
  if (!(out.f = fopen(path, "wb"))) return gbf_fail(GBF_ERR_ARG, "gbf_checkpoint_write: cannot open file");
  bool ok = fwrite(&step, sizeof(int), 1, out.f) == 1;
  ok = ok && fwrite(P1, sizeof(double), n, out.f) == n;
  ok = ok && fwrite(S2, sizeof(double), n, out.f) == n;
  for (int axis = 0; axis < 3 && ok; axis++) {
    coordinates(m, axis, xyz);
    ok = fwrite(xyz.data(), sizeof(double), n, out.f) == n;
  }
  if ((!roS1_old || !roS2_old) && zeros.empty()) zeros.assign(n, 0.0);
  ok = ok && fwrite(roS1_old ? roS1_old : zeros.data(), sizeof(double), n, out.f) == n;
  ok = ok && fwrite(roS2_old ? roS2_old : zeros.data(), sizeof(double), n, out.f) == n;
  if (media) {
    ok = ok && fwrite(media, sizeof(int), n, out.f) == n;
  } else {
    std::vector<int> zi(n, 0);
    ok = ok && fwrite(zi.data(), sizeof(int), n, out.f) == n;
  }
  ok = (fflush(out.f) == 0) && ok;
  return ok ? GBF_OK : gbf_fail(GBF_ERR_ARG, "gbf_checkpoint_write: short write");
}

int gbf_checkpoint_read(const char* path, const gbf_model* m, int* step, double* P1, double* S2, double* roS1_old,
                        double* roS2_old, int* media) {
  if (!path || !m || gbf_checkpoint_bytes(m) == 0) return gbf_fail(GBF_ERR_ARG, "gbf_checkpoint_read");
  const size_t n = cells_of(m);
  File in;
  if (!(in.f = fopen(path, "rb"))) return gbf_fail(GBF_ERR_ARG, "gbf_checkpoint_read: cannot open file");
  if (fseek(in.f, 0, SEEK_END) != 0) return gbf_fail(GBF_ERR_ARG, "gbf_checkpoint_read: seek");
  const long size = ftell(in.f);
  if (size < 0 || (size_t)size != gbf_checkpoint_bytes(m))
    return gbf_fail(GBF_ERR_ARG, "gbf_checkpoint_read: file size does not match the model's grid");
  rewind(in.f);
  int j = 0;
  std::vector<double> buf(n), want;
  auto field = [&](double* dst) -> bool {
    double* p = dst ? dst : buf.data();
    return fread(p, sizeof(double), n, in.f) == n;
  };
  bool ok = fread(&j, sizeof(int), 1, in.f) == 1;
  ok = ok && field(P1) && field(S2);
  for (int axis = 0; axis < 3 && ok; axis++) {
    ok = field(nullptr);
    coordinates(m, axis, want);
    if (ok && memcmp(buf.data(), want.data(), n * sizeof(double)) != 0)
      return gbf_fail(GBF_ERR_ARG, "gbf_checkpoint_read: cell coordinates do not match the model");
  }
  ok = ok && field(roS1_old) && field(roS2_old);
  if (ok) {
    std::vector<int> mi;
    int* dst = media;
    if (!dst) {
      mi.resize(n);
      dst = mi.data();
    }
    ok = fread(dst, sizeof(int), n, in.f) == n;
  }
  if (!ok) return gbf_fail(GBF_ERR_ARG, "gbf_checkpoint_read: short read");
  if (step) *step = j;
  return GBF_OK;
}

}  // extern "C"
