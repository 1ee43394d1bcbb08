/*
 * gbflow_dropin.h — the reference's GPU host function set, implemented by
 * libgbflow.so with C++ linkage so that the reference driver (main.cpp) and
 * its single-domain communication layer (no_communication.cpp) link against
 * it unchanged, in place of gpu.cu.
 *
 * The two structs repeat the reference's declarations (defines.h:41-61) with
 * the same tags, member order and types: the mangled names of the functions
 * below contain the tags, and the functions take the structs by value, so
 * both must match for link and call compatibility.
 *
 * A translation unit must include either this header or the reference's
 * defines.h, not both.
 */
#ifndef GBFLOW_DROPIN_H
#define GBFLOW_DROPIN_H

#ifdef __cplusplus

struct ptr_Arrays_tag {                       /* defines.h:41-46 */
  double *x, *y, *z;
  double *P1, *P2, *S2, *ro1, *ro2, *u1x, *u1y, *u1z, *u2x, *u2y, *u2z, *Xi1, *Xi2, *roS1, *roS1_old, *roS2, *roS2_old;
  int* media;
};
typedef struct ptr_Arrays_tag ptr_Arrays;      /* defines.h:47 */

struct consts_tag {                           /* defines.h:50-60 */
  double K[2];
  double lambda[2];
  double S_wr[2];
  double m[2];
  double P_d[2];
  double h1, h2, h3, dt, tau, l_w, l_n, c, beta1, beta2;
  int NX, Ny, Nz;
  int source, save_plots, print_screen;
};
typedef struct consts_tag consts;              /* defines.h:61 */

/* Hot path (replaces gpu.cu:87, :185, :335, :377, :474). */
void ro_P2_Xi_calculation(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, consts def, int localNx, int rank, int size, int blocksX, int blocksY, int blocksZ);  /* defines.h:106 */
void u_calculation(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, int localNx, int rank, int size, int blocksX, int blocksY, int blocksZ, consts def);          /* defines.h:108 */
void roS_calculation(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, consts def, double t, int localNx, int rank, int size, int blocksX, int blocksY, int blocksZ); /* defines.h:110 */
void P1_S2_calculation(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, consts def, int localNx, int rank, int size, int blocksX, int blocksY, int blocksZ);     /* defines.h:111 */
void boundary_conditions(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, int localNx, int rank, int size, int blocksX, int blocksY, int blocksZ, consts def);    /* defines.h:112 */

/* Data movement and device set-up (replaces gpu.cu:483-610). */
void load_data_to_host(double* HostArrayPtr, double* DevArrayPtr, int localNx, consts def);      /* defines.h:78 */
void load_data_to_device(double* HostArrayPtr, double* DevArrayPtr, int localNx, consts def);    /* defines.h:79 */
void load_data_to_device_int(int* HostArrayPtr, int* DevArrayPtr, int localNx, consts def);      /* defines.h:80 */
void device_memory_alloc(ptr_Arrays* ArraysPtr, double** DevBuffer, int nX, consts def);          /* defines.h:68 */
void device_memory_free(ptr_Arrays DevArraysPtr, double* DevBuffer);                                 /* defines.h:71 */
void Device_Initialize(int rank, int* blocksX, int* blocksY, int* blocksZ, int localNx, consts def); /* defines.h:82 */

/* Halo pack/unpack of the multi-rank layer (replaces gpu.cu:626, :648). */
void load_exchange_data(double* HostArrayPtr, double* DevArrayPtr, double* HostBuffer, double* DevBuffer, int localNx, int blocksY, int blocksZ, int rank, int size, consts def); /* defines.h:115 */
void save_exchange_data(double* HostArrayPtr, double* DevArrayPtr, double* HostBuffer, double* DevBuffer, int localNx, int blocksY, int blocksZ, int rank, int size, consts def); /* defines.h:116 */

#endif /* __cplusplus */

/* Extension entry points of the drop-in (C linkage). */
#ifdef __cplusplus
extern "C" {
#endif
/* 0 = eager (one kernel per reference function, reference intermediate
   arrays written by every call; the default), 1 = fused (the five calls of a
   step are deferred and run as one fused FP64 step at boundary_conditions;
   intermediate arrays are materialised on demand by load_data_to_host),
   2 = split (as 1, with the step in the headline split form: FP32 state and
   fluxes, FP64-precision masses and one residual-correction Newton step per
   cell, kept beside the caller's arrays; P1 and S2 are written back when the
   host reads them; results within the split form's bars, max|dS| <= 1e-5 and
   rel-L2(P) <= 1e-6, of the reference arithmetic). A process starts in mode
   1 or 2 when its environment holds GBF_DROPIN_MODE=1 or 2, so that a driver
   which cannot call this function (the reference's main.cpp) can select it.
   Changing the mode brings every caller array up to date first. */
int gbf_dropin_set_mode(int mode);
int gbf_dropin_get_mode(void);
/* The gbflow domain behind arrays from device_memory_alloc (keyed by their
   device P1 pointer) in fused or split mode, once the first step created it; NULL
   otherwise. It accepts the gbf_domain_* timing and status calls of
   gbflow.h (gbf_domain_set_timing, gbf_domain_kernel_times,
   gbf_domain_status); the drop-in owns it and frees it in
   device_memory_free. No counterpart in the reference. */
struct gbf_domain* gbf_dropin_domain(const double* dev_P1);
#ifdef __cplusplus
}
#endif

#endif /* GBFLOW_DROPIN_H */
