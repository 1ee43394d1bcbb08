// gbf_plots.cpp — the reference's Tecplot output, host side.
//
// save_data_plots (main.cpp:319-339) writes, for time t, five point-format
// Tecplot files and media.dat: the headers of print_plots_top
// (main.cpp:341-410) followed by the data of print_plots (main.cpp:412-482).
// This writer produces the same bytes for a single domain (rank 0 of 1, where
// every point is active and the global index I equals i), including the
// layout's particulars: the S2_x profile starts at cell (nx * ny) / 2 of each
// k plane, the vertical velocity is written as (-1) * u2y, and the heights are
// ny * h2 - y.
#include <errno.h>
#include <stdio.h>
#include <string.h>
#include <sys/stat.h>

#include <string>

#include "gbf_internal.h"

namespace {

struct Out {
  FILE* f = nullptr;
  ~Out() {
    if (f) fclose(f);
  }
};

bool make_dir(const std::string& p) { return mkdir(p.c_str(), 0777) == 0 || errno == EEXIST; }

}  // namespace

extern "C" int gbf_write_plots(const char* dir, const gbf_model* m, double t, const double* P1, const double* S2,
                               const double* u2x, const double* u2y, const double* u2z, const int* media) {
  if (!dir || !m || !P1 || !S2 || !u2x || !u2y || !u2z || m->nx < 1 || m->ny < 1 || m->nz < 1)
    return gbf_fail(GBF_ERR_ARG, "gbf_write_plots");
  const int nx = m->nx, ny = m->ny, nz = m->nz;
  const std::string root = std::string(dir) + "/";
  for (const char* sub : {"plot_P1", "plot_S2", "plot_u", "plot_S2_y", "plot_S2_x"})
    if (!make_dir(root + sub)) return gbf_fail(GBF_ERR_ARG, "gbf_write_plots: cannot create directory");
  char name[5][64];
  snprintf(name[0], sizeof(name[0]), "plot_S2/S2=%012.4f.dat", t);
  snprintf(name[1], sizeof(name[1]), "plot_P1/P1=%012.4f.dat", t);
  snprintf(name[2], sizeof(name[2]), "plot_u/u=%012.4f.dat", t);
  snprintf(name[3], sizeof(name[3]), "plot_S2_y/S2=%012.4f.dat", t);
  snprintf(name[4], sizeof(name[4]), "plot_S2_x/S2=%012.4f.dat", t);
  Out S2f, P1f, uf, S2y, S2x, mf;
  Out* files[5] = {&S2f, &P1f, &uf, &S2y, &S2x};
  for (int q = 0; q < 5; q++)
    if (!(files[q]->f = fopen((root + name[q]).c_str(), "w"))) return gbf_fail(GBF_ERR_ARG, "gbf_write_plots: open");
  if (!(mf.f = fopen((root + "media.dat").c_str(), "w"))) return gbf_fail(GBF_ERR_ARG, "gbf_write_plots: open");

  // headers (print_plots_top)
  fprintf(S2f.f, "TITLE =  \"Saturation of DNALP in time=%5.2f\" \n", t);
  fprintf(S2f.f, "VARIABLES = \"X\",\"Y\",\"Z\",\"S2\",\"P1\",\"u_x\", \"u_y\", \"u_z\" \n");
  fprintf(S2f.f, "ZONE T = \"BIG ZONE\", K=%d,J=%d,I=%d, F = POINT\n", nx, nz, ny);
  fprintf(P1f.f, "TITLE =  \"Pressure of water in time=%5.2f\" \n", t);
  fprintf(P1f.f, "VARIABLES = \"X\",\"Y\",\"P1\" \n");
  fprintf(P1f.f, "ZONE T = \"BIG ZONE\", J=%d,I=%d, F = POINT\n", nx, ny);
  fprintf(uf.f, "TITLE =  \"Velocity of DNALP in time=%5.2f\" \n", t);
  fprintf(uf.f, "VARIABLES = \"X\",\"Y\",\"u_x\", \"u_y\" \n");
  fprintf(uf.f, "ZONE T = \"BIG ZONE\", J=%d,I=%d, F = POINT\n", nx - 2, ny - 2);
  fprintf(S2y.f, "TITLE =  \"Saturation of DNALP in time=%5.2f\" \n", t);
  fprintf(S2y.f, "VARIABLES = \"Y\",\"S2\" \n");
  fprintf(S2y.f, "ZONE T = \"BIG ZONE\", J=%d, F = POINT\n", ny);
  fprintf(S2x.f, "TITLE =  \"Saturation of DNALP in time=%5.2f\" \n", t);
  fprintf(S2x.f, "VARIABLES = \"X\",\"S2\" \n");
  fprintf(S2x.f, "ZONE T = \"BIG ZONE\", J=%d, F = POINT\n", nx);
  fprintf(mf.f, "TITLE =  \"Porous media\" \n");
  fprintf(mf.f, "VARIABLES = \"X\",\"Y\",\"media\" \n");
  fprintf(mf.f, "ZONE T = \"BIG ZONE\", J=%d,I=%d, F = POINT\n", nx, ny);

  // data (print_plots); coordinates as initial_data sets them (main.cpp:115-117)
  const size_t pl = (size_t)nx * ny;
  auto X = [&](size_t c) { return (double)(int)(c % nx) * (m->h1); };
  auto Y = [&](size_t c) { return (double)(int)((c / nx) % ny) * (m->h2); };
  auto Z = [&](size_t c) { return (double)(int)(c / pl) * (m->h3); };
  const double H = ny * (m->h2);
  for (int i = 0; i < nx; i++)
    for (int j = 0; j < ny; j++)
      for (int k = 0; k < nz; k++) {
        const size_t c = (size_t)i + (size_t)j * nx + (size_t)k * pl;
        fprintf(S2f.f, "%.2e %.2e %.2e %.3e %.3e %.3e %.3e %.3e\n", X(c), Z(c), H - Y(c), S2[c], P1[c], u2x[c], u2z[c],
                (-1) * u2y[c]);
        fprintf(P1f.f, "%d %d %d %.3e %.3e %.3e %.3e %.3e\n", i, j, k, S2[c], P1[c], u2x[c], u2z[c], (-1) * u2y[c]);
        fprintf(mf.f, "%.2e %.2e %d\n", X(c), H - Y(c), media ? media[c] : 0);
        fprintf(uf.f, "%.2e %.2e %.3e %.3e\n", X(c), H - Y(c), u2x[c], (-1) * u2y[c]);
      }
  for (int i = 1; i < nx - 1; i++)
    for (int j = 1; j < ny - 1; j++)
      for (int k = 1; k < nz - 1; k++) {
        const size_t c = (size_t)i + (size_t)j * nx + (size_t)k * pl;
        fprintf(uf.f, "%.2e %.2e %.3e %.3e\n", X(c), H - Y(c), u2x[c], (-1) * u2y[c]);
      }
  for (int i = 0; i < nx; i++)
    for (int k = 0; k < nz; k++)
      if (i == nx / 2)
        for (int j = 0; j < ny; j++) {
          const size_t c = (size_t)(nx / 2) + (size_t)j * nx + (size_t)k * pl;
          fprintf(S2y.f, "%.2e %.3e\n", Y(c), S2[c]);
        }
  for (int i = 0; i < nx; i++)
    for (int k = 0; k < nz; k++) {
      const size_t c = (size_t)i + pl / 2 + (size_t)k * pl;
      fprintf(S2x.f, "%.2e %.3e\n", X(c), S2[c]);
    }
  bool ok = true;
  for (Out* o : {&S2f, &P1f, &uf, &S2y, &S2x, &mf}) ok = (fflush(o->f) == 0) && !ferror(o->f) && ok;
  return ok ? GBF_OK : gbf_fail(GBF_ERR_ARG, "gbf_write_plots: write error");
}
