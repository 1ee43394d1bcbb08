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
       GBF_PREC_SPLIT = 1,             /* FP32 P,S,K,fluxes; phase masses at least as precise
                                          as FP64: FP32-pair defects over the state's exact
                                          FP32-product mass; after the FP32 Newton step one
                                          residual-correction step per cell, its residual
                                          exact to FP64 precision by error-free FP32
                                          transformations (FP32 pipes only)              */
       GBF_PREC_SPLIT_DF = 2,          /* as SPLIT, masses and residual as FP32 pairs
                                          (about 48 significant bits, FP32 pipes only)  */
       GBF_PREC_SPLIT_DEFECT = 3 };    /* as SPLIT, each phase mass held as its FP32
                                          excess ("defect") over the mass the FP32 state
                                          gives at the row's hydrostatic density, an
                                          exact product: 4 bytes a phase and cell, the
                                          residual and mass update in FP32 on small
                                          numbers (FP32 pipes only)                     */

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
/* sizeof of the ABI structs (0: gbf_model, 1: gbf_cells, 2: gbf_arrays,
   3: gbf_run_defines), so bindings can check their layout. */
size_t gbf_abi_sizeof(int which);
/* Fill *m with the reference's constants (defines.h:6-26) and the defaults of
   its defines.ini; grid sizes nx, ny, nz and dt are taken from the arguments. */
void gbf_model_reference(gbf_model* m, int nx, int ny, int nz, double dt);
/* Largest stable explicit dt (times `safety`) for this model and cell fields.
   Pure host function; K/phi may be NULL (media table used). */
double gbf_stable_dt(const gbf_model* m, const gbf_cells* cells, double safety);
/* The reference's run parameters that gbf_model does not hold (consts,
   defines.h:50-61): the hyperbolic-regularisation constants of the unused
   t < 2 dt branch (tau, l_w, l_n, c) and main.cpp's output intervals. */
typedef struct gbf_run_defines {
  double tau, l_w, l_n, c;
  int save_plots, print_screen;
} gbf_run_defines;
/* Read a defines.ini file (the reference's format, main.cpp:601-684, from a
   path instead of defines.h:5's fixed Windows path): *m gets
   gbf_model_reference's values overridden by H1, H2, H3, DT, BETA1, BETA2,
   SOURCE, NX, NY, NZ and by the physical constants the file lists (K[i],
   LAMBDA[i], S_WR[i], M[i], P_D[i], MU1, MU2, RO_W, RO_N, S2_GR, P_ATM,
   G_CONST; the reference takes these from defines.h:6-26 instead, with the
   same values); *run (may be NULL) TAU, L_W, L_N, C, SAVE_PLOTS,
   PRINT_SCREEN. NX, NY and NZ are required. */
int gbf_read_defines(const char* path, gbf_model* m, gbf_run_defines* run);
/* Host-side validation of a model (sizes, positivity, S_e range of the Dirichlet
   patch, dt against the stability bound when check_dt != 0). */
int gbf_model_validate(const gbf_model* m, const gbf_cells* cells, int check_dt);

/* ------------------------------------------------ seeded synthetic fields
 * Host functions (no GPU). Deterministic for a seed, whatever the thread
 * count. K: log-normal, geometric mean K_geo, log-standard deviation
 * sigma_lnK, built from white noise smoothed by a Gaussian of corr_cells
 * cells and renormalised to unit variance. phi: base + amp * U(-1, 1).
 */
int gbf_fill_lognormal_K(int nx, int ny, int nz, uint64_t seed, double K_geo, double sigma_lnK, double corr_cells,
                         float* K_out);
int gbf_fill_porosity(int nx, int ny, int nz, uint64_t seed, double base, double amp, float* phi_out);
/* The same fields generated on the device into device arrays (enqueued on
   `stream`; the K generator returns after its work completed). Porosity is
   bit-identical to gbf_fill_porosity; K equals gbf_fill_lognormal_K up to the
   last-bit differences of the host's and the device's log, cos and exp, i.e.
   within 1 FP32 ulp, in all but a handful of cells bit for bit. */
int gbf_fill_lognormal_K_device(int nx, int ny, int nz, uint64_t seed, double K_geo, double sigma_lnK,
                                double corr_cells, float* d_K, void* stream);
int gbf_fill_porosity_device(int nx, int ny, int nz, uint64_t seed, double base, double amp, float* d_phi,
                             void* stream);

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
/* a5 for callers that cannot allocate device memory where they apply the
   boundary conditions: a host loop that must not stall on cudaMalloc (it
   synchronises the device), a process whose device memory belongs to another
   framework's caching allocator or is budgeted up front, a driver that hands
   over only its own state arrays and no workspace.
   No counterpart in the reference. Same results as gbf_boundary_f64; its
   scratch is a fixed 8 MiB array of the library in device memory that every
   GPU loading the library keeps until exit, so it serves grids with at most
   524288 boundary cells (2 nx ny + 2 nx (nz - 2) + 2 (ny - 2) (nz - 2): cubes
   up to 296^3) and returns GBF_ERR_ARG beyond, before any work.
   Allocates nothing. Its first call on a device, and its first call after
   that device's context was destroyed and created again, look up the array's
   device address, so make those calls before any stream capture. All calls
   share the array: calls that overlap on the GPU race. */
int gbf_boundary_f64_noalloc(const gbf_model* m, gbf_arrays d_arrays, void* stream);

/* ------------------------------------------------------- single domain ----
 * One grid whose state lives in HBM between steps. `precision` is
 * GBF_PREC_F64 (plain FP64: two passes per step — properties, then fluxes,
 * mass update and Newton fused — plus a face pass for the boundaries) or
 * GBF_PREC_SPLIT (FP32 P, S, K, phi and fluxes; per-cell phase masses at
 * least as precise as FP64, as FP32-pair defects), GBF_PREC_SPLIT_DF (the
 * masses and residual as FP32 pairs)
 * or GBF_PREC_SPLIT_DEFECT (the masses as FP32 defects). All
 * calls are ordered on the domain's
 * stream; gbf_domain_step only enqueues work.
 */
typedef struct gbf_domain gbf_domain;
typedef struct gbf_ensemble gbf_ensemble; /* batched grids, declared below */
/* Per-step outputs that are off by default (the hot path writes P, S only). */
enum { GBF_OUT_MASS = 1,        /* phase masses after the mass update, every step */
       GBF_OUT_VELOCITY = 2,    /* u1x..u2z of the reference's a2 (FP64 only)      */
       GBF_OUT_MASS_ARRAYS = 4, /* roS1, roS2, roS1_old, roS2_old (FP64 only)       */
       GBF_OUT_PROPS = 8,       /* keep P2/Xi/ro of the last step readable        */
       GBF_OUT_CFL = 16 };      /* with GBF_OUT_MASS, split forms: CFL numbers per
                                   step (cell maximum of face flux dt / (phi h) per phase) */
int gbf_domain_create(const gbf_model* m, const gbf_cells* host_cells, int precision, gbf_domain** out);
int gbf_domain_destroy(gbf_domain* d);
int gbf_domain_set_outputs(gbf_domain* d, int out_flags, int mass_history_capacity);
int gbf_domain_set_stream(gbf_domain* d, void* stream);
/* Initial state from host arrays (nx*ny*nz doubles each). */
int gbf_domain_upload(gbf_domain* d, const double* P1_host, const double* S2_host);
/* Same from device arrays (e.g. torch tensors). */
int gbf_domain_upload_device(gbf_domain* d, const double* P1_dev, const double* S2_dev);
int gbf_domain_step(gbf_domain* d, int nsteps);
/* Copy one field (GBF_FIELD_*) of the current state to the host; synchronises. */
int gbf_domain_download(gbf_domain* d, int field, double* host);
/* Host-resident grid in one call: upload(P_in, S_in), `nsteps` steps,
   download of P1 into P_out and S2 into S_out. For one step of a split-
   precision grid without a Dirichlet patch, of 2M cells or more, it is
   pipelined over slabs of planes (about 1M cells each, at most 16) on three
   streams (host-to-device copies; conversion, the step's
   chunk layer and the boundary rules of each slab; device-to-host copies),
   so that the two copy directions overlap; otherwise the three calls in
   turn. The outputs may alias the inputs. The state equals the three calls'
   bit for bit; the step's phase masses (GBF_OUT_MASS) sum the same cells in
   other partial blocks (within 1e-11 relative). Overlap needs page-locked
   host arrays. Returns after the last copy. */
int gbf_domain_advance_host(gbf_domain* d, const double* P_in, const double* S_in, int nsteps, double* P_out,
                            double* S_out);
/* Phase masses [step][2] recorded since the last upload (GBF_OUT_MASS). */
int gbf_domain_mass_history(gbf_domain* d, double* host, int max_steps, int* nsteps_out);
/* CFL numbers [step][2] (water, DNAPL) of the same steps (GBF_OUT_CFL): the
   largest over interior cells and their six faces of the phase's volumetric
   face flux (mass flux / reference density) times dt / (phi h). */
int gbf_domain_cfl_history(gbf_domain* d, float* host, int max_steps, int* nsteps_out);
/* Synchronise and return the device-side status (non-finite P/S, timeouts). */
int gbf_domain_status(gbf_domain* d);
int gbf_domain_sync(gbf_domain* d);
long long gbf_domain_steps_done(gbf_domain* d);
/* Kernels launched per step (for launch accounting). */
int gbf_domain_launches_per_step(gbf_domain* d);
/* Per-kernel CUDA-event timing on the domain's stream (off by default):
   gbf_domain_kernel_times synchronises, returns milliseconds and launch
   counts per kernel kind (gbf_kernel_name) since the last call, and resets. */
int gbf_domain_set_timing(gbf_domain* d, int on);
int gbf_domain_kernel_times(gbf_domain* d, double* ms, int* launches, int nkinds);
int gbf_kernel_kinds(void);
const char* gbf_kernel_name(int kind);
/* Split kernels stage their x-y planes by TMA (cp.async.bulk.tensor) where a
   grid qualifies (FP32 K field, no media table, nx % 4 == 0), else by plain
   loads. 0 forces plain loads for domains and ensembles created afterwards
   (and ensemble tile lists rebuilt afterwards); default 1. Negative `on`
   leaves the setting as it is. Returns the setting in force before the call. */
int gbf_set_tma(int on);
/* Host arrays that are page-locked (cudaHostAlloc, cudaHostRegister) are read
   and written in place by the FP64 <-> split conversion kernels of the upload
   and download calls (split-precision domains and ensembles), over the
   CPU-GPU link, instead of being staged through device memory by copies.
   0 forces staging; negative leaves the setting as it is; default 1. Returns
   the setting in force before the call. */
int gbf_set_host_direct(int on);
/* Diagnostic of the device-side failure detection: one block runs the TMA
   tiles' bounded mbarrier wait on a barrier phase that never completes, with
   `tries` rounds; it must give up and report GBF_ERR_TIMEOUT (no trap, the
   context stays usable). *ms (may be NULL) receives the kernel's time. The
   tiles use 2^18 rounds per wait (about 1 s on GB300). */
int gbf_diag_bounded_wait(unsigned tries, double* ms);
/* 1 if the object's split step stages planes by TMA, 0 if by plain loads. */
int gbf_domain_uses_tma(gbf_domain* d);
int gbf_ensemble_uses_tma(gbf_ensemble* e);

/* ------------------------------------------------------------ checkpoints
 * The reference's checkpoint file save/save.dat (main.cpp:485-572), one
 * domain: int step; double P1, S2, x, y, z, roS1_old, roS2_old; int media;
 * n = nx*ny*nz values each, index i + j*nx + k*nx*ny, native byte order.
 * x, y, z are the cell coordinates i*h1, j*h2, k*h3 (main.cpp:115-117); the
 * reader refuses a file whose size or coordinates do not match the model.
 * CPU-written checkpoints restore into GPU domains and back.
 */
size_t gbf_checkpoint_bytes(const gbf_model* m);
/* NULL roS1_old/roS2_old/media are written as zeros. */
int gbf_checkpoint_write(const char* path, const gbf_model* m, int step, const double* P1, const double* S2,
                         const double* roS1_old, const double* roS2_old, const int* media);
/* NULL outputs are skipped. */
int gbf_checkpoint_read(const char* path, const gbf_model* m, int* step, double* P1, double* S2, double* roS1_old,
                        double* roS2_old, int* media);
/* The domain's state as such a file. roS1_old/roS2_old are those the
   reference holds after its last step: start-of-step phase masses of the
   interior cells (cpu.cpp:222-225, 286-287), computed from the state before
   that step (zeros before the first step); media is the domain's table index
   (zeros without one). */
int gbf_domain_save(gbf_domain* d, const char* path, int step);
/* Upload (P1, S2) from such a file, after checking that its media equal the
   domain's; *step receives the file's step. */
int gbf_domain_restore(gbf_domain* d, const char* path, int* step);

/* ------------------------------------------------------------ plot files
 * The reference's Tecplot output of save_data_plots (main.cpp:319-482) for
 * one domain, written under `dir`: plot_S2/S2=<t>.dat, plot_P1/P1=<t>.dat,
 * plot_u/u=<t>.dat, plot_S2_y/S2=<t>.dat, plot_S2_x/S2=<t>.dat (t as
 * %012.4f) and media.dat, byte for byte as the reference writes them from
 * the same arrays. Subdirectories are created; a NULL media writes 0.
 */
int gbf_write_plots(const char* dir, const gbf_model* m, double t, const double* P1, const double* S2,
                    const double* u2x, const double* u2y, const double* u2z, const int* media);
/* The domain's state: P1, S2 as downloaded and the DNAPL velocities the
   reference holds after its last step (those of the state that step started
   from; zeros before the first step). */
int gbf_domain_write_plots(gbf_domain* d, const char* dir, double t);

/* ----------------------------------------------------------- ensembles ----
 * Independent realizations of uneven sizes and parameters, advanced
 * together: every gbf_ensemble_step moves every member by one of its own
 * time steps. Split precisions run one persistent kernel over a packed tile
 * work list of all members; FP64 runs its two passes over packed chunk
 * lists. Each step is a CUDA graph. `host_cells` may be NULL or an array of
 * n entries. Uploads and downloads are per member (FP64 host or device
 * arrays of nx*ny*nz doubles).
 */
int gbf_ensemble_create(int n, const gbf_model* models, const gbf_cells* host_cells, int precision,
                        gbf_ensemble** out);
int gbf_ensemble_destroy(gbf_ensemble* e);
int gbf_ensemble_size(gbf_ensemble* e);
long long gbf_ensemble_cells(gbf_ensemble* e);
long long gbf_ensemble_interior_cells(gbf_ensemble* e);
int gbf_ensemble_set_stream(gbf_ensemble* e, void* stream);
/* GBF_OUT_MASS only: per-member phase masses every step. */
int gbf_ensemble_set_outputs(gbf_ensemble* e, int out_flags, int mass_history_capacity);
/* GBF_OUT_CFL (with GBF_OUT_MASS, split forms): [step][member][2] CFL numbers,
   as gbf_domain_cfl_history. */
int gbf_ensemble_cfl_history(gbf_ensemble* e, float* host, int max_steps, int* nsteps_out);
int gbf_ensemble_upload(gbf_ensemble* e, int member, const double* P1, const double* S2);
/* Every member at once: P_all and S_all hold all members' nx*ny*nz doubles
   back to back in member order (host or device memory; pinned host memory
   moves at full link speed). Both return after the transfer completed. */
int gbf_ensemble_upload_all(gbf_ensemble* e, const double* P_all, const double* S_all);
int gbf_ensemble_download_all(gbf_ensemble* e, double* P_all, double* S_all);
/* Host-resident ensemble in one call: upload_all(P_in, S_in), `nsteps`
   steps, download_all(P_out, S_out), pipelined over groups of members on
   three streams (host-to-device copies, conversion and steps, device-to-host
   copies) so that the two copy directions and the steps of different groups
   overlap. The outputs may alias the inputs. Results equal the three calls
   bit for bit; phase masses are not recorded (the mass history restarts
   empty). Overlap needs page-locked host arrays. Returns after the last copy. */
int gbf_ensemble_advance_host(gbf_ensemble* e, const double* P_in, const double* S_in, int nsteps, double* P_out,
                              double* S_out);
/* Member groups of gbf_ensemble_advance_host (1..16, at most one per member);
   0 (default): about 4M cells per group. */
int gbf_ensemble_set_pipeline_groups(gbf_ensemble* e, int groups);
int gbf_ensemble_step(gbf_ensemble* e, int nsteps);
int gbf_ensemble_download(gbf_ensemble* e, int member, int field, double* host);
/* [step][member][2] since the last upload. */
int gbf_ensemble_mass_history(gbf_ensemble* e, double* host, int max_steps, int* nsteps_out);
int gbf_ensemble_status(gbf_ensemble* e);
int gbf_ensemble_sync(gbf_ensemble* e);
int gbf_ensemble_set_timing(gbf_ensemble* e, int on);
int gbf_ensemble_kernel_times(gbf_ensemble* e, double* ms, int* launches, int nkinds);
int gbf_ensemble_launches_per_step(gbf_ensemble* e);
/* Tuning: tile shape (0: 32x8, 1: 64x4, 2: 32x4, 3: 64x8 and 4: 32x16 cells
   with two cells per thread, 5: 32x16 with a 48x10 tile ending the rows of
   grids whose nx is 16 more than a multiple of 32 — the last three need TMA
   staging: GBF_ERR_ARG without it; -1 keeps it) and the k planes
   per tile pass ("fusion depth") of members whose nx == edge (0: whole column).
   gbf_ensemble_autotune times `trial_steps` steps per candidate and keeps the
   fastest; it advances the state, so upload the initial state afterwards. */
int gbf_ensemble_set_tuning(gbf_ensemble* e, int shape, int edge, int kchunk);
int gbf_ensemble_get_tuning(gbf_ensemble* e, int* shape, int* edges, int* kchunks, int max_entries);
const char* gbf_ensemble_shape_name(int shape);
int gbf_ensemble_autotune(gbf_ensemble* e, int trial_steps);

#ifdef __cplusplus
}
#endif
#endif /* GBFLOW_H */
