/*
 * gbflow.h — C ABI of the GB300 hot path for the two-phase water/DNAPL
 * porous-media flow step (Darcy face fluxes, explicit phase-mass update,
 * per-cell Newton (P, S) recovery, boundary conditions).
 *
 * Grid convention (same as the reference, defines.h:41-47, cpu.cpp:59):
 *   cell index c = i + j*nx + k*nx*ny; i = x (fastest), j = vertical
 *   (gravity acts along +j, j = 0 is the top), k = z (slowest).
 *
 * Every function returns a gbf status code (GBF_OK on success) unless noted.
 * No torch types appear here: plain pointers, sizes and POD structs only.
 *
 * The reference's own host function set (defines.h:63-116, C++ linkage) is
 * declared separately in gbflow_dropin.h; it is implemented on top of this ABI.
 */
#ifndef GBFLOW_H
#define GBFLOW_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  GBF_OK = 0,
  GBF_ERR_ARG = 1,        /* bad argument / unsupported size               */
  GBF_ERR_CUDA = 2,       /* a CUDA runtime call failed                     */
  GBF_ERR_NOMEM = 3,      /* device allocation failed                       */
  GBF_ERR_NONFINITE = 4,  /* a NaN/Inf appeared in P or S on the device     */
  GBF_ERR_UNSTABLE = 5,   /* dt above the explicit-scheme stability bound   */
  GBF_ERR_TIMEOUT = 6,    /* a bounded device-side wait gave up             */
  GBF_ERR_STATE = 7       /* call out of order (e.g. step before upload)    */
};

/* --------------------------------------------------------------- options */
enum { GBF_SOURCE_DIRICHLET_PATCH = 0, /* reference: S2 = S2_gr on the top patch */
       GBF_SOURCE_RATE = 1 };          /* mass-rate injection into top interior cells */
enum { GBF_BC_REFERENCE = 0,           /* reference Border_S2/Border_P1 rules           */
       GBF_BC_HYDROSTATIC_SIDES = 1 }; /* Dirichlet hydrostatic P on i/k sides,
                                          no-flow bottom face for both phases          */
enum { GBF_PREC_F64 = 0,               /* plain FP64 state and arithmetic               */
       GBF_PREC_SPLIT = 1 };           /* FP32 P,S,K,fluxes; FP64 phase masses and residual */

/* Fields that can be read back (gbf_domain_download / ensemble download). */
enum {
  GBF_FIELD_P1 = 0, GBF_FIELD_S2, GBF_FIELD_P2, GBF_FIELD_RO1, GBF_FIELD_RO2,
  GBF_FIELD_XI1, GBF_FIELD_XI2, GBF_FIELD_U1X, GBF_FIELD_U1Y, GBF_FIELD_U1Z,
  GBF_FIELD_U2X, GBF_FIELD_U2Y, GBF_FIELD_U2Z, GBF_FIELD_ROS1, GBF_FIELD_ROS2,
  GBF_FIELD_ROS1_OLD, GBF_FIELD_ROS2_OLD, GBF_FIELD_COUNT
};

/*
 * Model parameters. The first block is the reference's `consts` (defines.h:50-61)
 * plus its compile-time physics macros (defines.h:6-26) made runtime values;
 * the second block holds extensions whose zero/one values give the reference's
 * behaviour exactly.
 */
typedef struct gbf_model {
  int nx, ny, nz;                 /* NX, Ny, Nz */
  double h1, h2, h3, dt;          /* cell sizes [m], time step [s] */
  double K[2], lambda[2], S_wr[2], m[2], P_d[2];  /* per-media table */
  double beta1, beta2;            /* compressibilities [1/Pa] */
  double mu1, mu2, ro01, ro02;    /* viscosities [Pa s], reference densities */
  double S2_gr, P_atm, g;         /* Dirichlet patch saturation, top pressure, gravity */
  int source;                     /* half-width of the Dirichlet patch */
  int newton_iterations;          /* reference: 7 (defines.h:15) */
  /* ---- extensions ---- */
  int source_mode;                /* GBF_SOURCE_* */
  int rate_cells;                 /* n: injection over an n x n patch (rate mode) */
  double rate;                    /* total DNAPL injection rate [kg/s] (rate mode) */
  int bc_mode;                    /* GBF_BC_* */
  double kv;                      /* vertical/horizontal permeability ratio (1 = isotropic) */
  double newton_tol;              /* 0: always run newton_iterations (reference);
                                     >0: stop once |dS| and |dP|/P_atm fall below it */
} gbf_model;

/*
 * Per-cell inputs. Either `media` (index into the model's 2-entry table, as in
 * the reference) or per-cell `K`/`phi` (FP32; FP64 paths promote them exactly).
 * A NULL K/phi falls back to the media table; a NULL media means media 0.
 */
typedef struct gbf_cells {
  const int* media;
  const float* K;
  const float* phi;
} gbf_cells;

/* Full set of reference state/derived arrays (ptr_Arrays, defines.h:41-47). */
typedef struct gbf_arrays {
  double *P1, *P2, *S2, *ro1, *ro2, *u1x, *u1y, *u1z, *u2x, *u2y, *u2z;
  double *Xi1, *Xi2, *roS1, *roS1_old, *roS2, *roS2_old;
} gbf_arrays;

/* ------------------------------------------------------------ utilities */
int gbf_last_status(void);            /* sticky status of the last failing call */
void gbf_clear_status(void);
const char* gbf_status_string(int status);
const char* gbf_version(void);
/* Fill *m with the reference's constants (defines.h:6-26) and the defaults of
   its defines.ini; grid sizes nx, ny, nz and dt are taken from the arguments. */
void gbf_model_reference(gbf_model* m, int nx, int ny, int nz, double dt);
/* Largest stable explicit dt (times `safety`) for this model and cell fields.
   Pure host function; K/phi may be NULL (media table used). */
double gbf_stable_dt(const gbf_model* m, const gbf_cells* cells, double safety);
/* Host-side validation of a model (sizes, positivity, S_e range of the Dirichlet
   patch, dt against the stability bound when check_dt != 0). */
int gbf_model_validate(const gbf_model* m, const gbf_cells* cells, int check_dt);

/* --------------------------- per-function device entry points (FP64) ----
 * Device pointers (`d_arrays`, `d_cells`), one CUDA stream (NULL = legacy
 * default stream). Asynchronous: they enqueue kernels and return. These are
 * the kernels behind the reference's five hot-path functions.
 */
int gbf_props_f64(const gbf_model* m, gbf_arrays d_arrays, gbf_cells d_cells, void* stream);     /* a1 */
int gbf_velocity_f64(const gbf_model* m, gbf_arrays d_arrays, void* stream);                      /* a2 */
int gbf_mass_f64(const gbf_model* m, gbf_arrays d_arrays, gbf_cells d_cells, void* stream);      /* a3 */
int gbf_newton_f64(const gbf_model* m, gbf_arrays d_arrays, gbf_cells d_cells, void* stream);    /* a4 */
/* a5; `d_scratch` must hold gbf_boundary_scratch_doubles(m) doubles (device). */
int gbf_boundary_f64(const gbf_model* m, gbf_arrays d_arrays, double* d_scratch, void* stream);
size_t gbf_boundary_scratch_doubles(const gbf_model* m);

#ifdef __cplusplus
}
#endif
#endif /* GBFLOW_H */
