// ref_shim.cpp — TEST INFRASTRUCTURE ONLY (part of the oracle).
//
// Thin extern "C" entry points over the reference's own CPU backend, compiled
// unmodified from its sources (cpu.cpp, main.cpp, no_communication.cpp) by
// oracle/Makefile into oracle/_ref/. Used to pin the C restatement
// (gbf_oracle.c) and to generate the golden fixtures under tests/golden/.
//
// Array order of `arrs` (20 pointers) is ptr_Arrays' field order
// (defines.h:41-47): x, y, z, P1, P2, S2, ro1, ro2, u1x, u1y, u1z, u2x, u2y,
// u2z, Xi1, Xi2, roS1, roS1_old, roS2, roS2_old.
#include "defines.h"

static ptr_Arrays make_arrays(double** a, int* media) {
  ptr_Arrays p;
  p.x = a[0]; p.y = a[1]; p.z = a[2];
  p.P1 = a[3]; p.P2 = a[4]; p.S2 = a[5]; p.ro1 = a[6]; p.ro2 = a[7];
  p.u1x = a[8]; p.u1y = a[9]; p.u1z = a[10]; p.u2x = a[11]; p.u2y = a[12]; p.u2z = a[13];
  p.Xi1 = a[14]; p.Xi2 = a[15]; p.roS1 = a[16]; p.roS1_old = a[17]; p.roS2 = a[18]; p.roS2_old = a[19];
  p.media = media;
  return p;
}

extern "C" {

int ref_sizeof_consts(void) { return (int)sizeof(consts); }

// main.cpp:97 initial_data on a single domain (rank 0, size 1).
void ref_initial_data(double** arrs, int* media, const consts* def) {
  ptr_Arrays H = make_arrays(arrs, media);
  int t = 0;
  initial_data(H, &t, def->NX, def->Ny, 0, 1, *def);
}

// main.cpp:83 time_step_function, `nsteps` times (single domain).
void ref_time_steps(double** arrs, int* media, const consts* def, int nsteps) {
  ptr_Arrays H = make_arrays(arrs, media);
  for (int s = 1; s <= nsteps; s++)
    time_step_function(H, H, 0, *def, s * def->dt, def->NX, def->Ny, 0, 1, 0, 0, 0);
}

// The five hot-path functions of cpu.cpp, one call each.
void ref_ro_P2_Xi(double** arrs, int* media, const consts* def) {
  ptr_Arrays H = make_arrays(arrs, media);
  ro_P2_Xi_calculation(H, H, *def, def->NX, 0, 1, 0, 0, 0);
}
void ref_u(double** arrs, int* media, const consts* def) {
  ptr_Arrays H = make_arrays(arrs, media);
  u_calculation(H, H, def->NX, 0, 1, 0, 0, 0, *def);
}
void ref_roS(double** arrs, int* media, const consts* def, double t) {
  ptr_Arrays H = make_arrays(arrs, media);
  roS_calculation(H, H, *def, t, def->NX, 0, 1, 0, 0, 0);
}
void ref_P1_S2(double** arrs, int* media, const consts* def) {
  ptr_Arrays H = make_arrays(arrs, media);
  P1_S2_calculation(H, H, *def, def->NX, 0, 1, 0, 0, 0);
}
void ref_boundary(double** arrs, int* media, const consts* def) {
  ptr_Arrays H = make_arrays(arrs, media);
  boundary_conditions(H, H, def->NX, 0, 1, 0, 0, 0, *def);
}

}  // extern "C"

// main.cpp:485 save / main.cpp:541 restore (single domain). Both work on
// "save/save.dat" relative to the working directory, so the call runs in
// `dir` and returns to the previous working directory afterwards.
#include <limits.h>
#include <unistd.h>

extern "C" int ref_save(const char* dir, double** arrs, int* media, const consts* def, int j) {
  char prev[PATH_MAX];
  if (!getcwd(prev, sizeof(prev)) || chdir(dir) != 0) return -1;
  ptr_Arrays H = make_arrays(arrs, media);
  save(H, H, j, 0, 1, def->NX, *def);
  return chdir(prev);
}

extern "C" int ref_restore(const char* dir, double** arrs, int* media, const consts* def, int* j) {
  char prev[PATH_MAX];
  if (!getcwd(prev, sizeof(prev)) || chdir(dir) != 0) return -1;
  ptr_Arrays H = make_arrays(arrs, media);
  restore(H, j, 0, 1, def->NX, *def);
  return chdir(prev);
}

// main.cpp:319 save_data_plots (single domain), run in `dir`: writes the
// Tecplot files plot_*/...=<t>.dat and media.dat there.
extern "C" int ref_plots(const char* dir, double** arrs, int* media, const consts* def, double t) {
  char prev[PATH_MAX];
  if (!getcwd(prev, sizeof(prev)) || chdir(dir) != 0) return -1;
  ptr_Arrays H = make_arrays(arrs, media);
  save_data_plots(H, H, t, 1, 0, def->NX, *def);
  return chdir(prev);
}
