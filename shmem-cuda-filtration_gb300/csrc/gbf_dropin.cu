// gbf_dropin.cu — the reference's GPU host function set (defines.h:63-116,
// C++ linkage) on top of the gbflow C ABI. The reference driver main.cpp and
// no_communication.cpp link against libgbflow.so in place of gpu.cu.
//
// Differences from gpu.cu that are deliberate:
//   * kernels cover the whole grid for every size (gpu.cu:61-62 does not);
//   * the Newton step runs the CPU path's 7 iterations (cpu.cpp:300);
//   * boundary values follow the CPU path's sweep order (cpu.cpp:44-54);
//   * no device-wide synchronisation after every launch (gpu.cu:9-26 syncs
//     under TEST): launches are ordered on the legacy default stream and the
//     blocking copies of load_data_to_host synchronise;
//   * errors are printed like checkErrors (gpu.cu:7-27) and also kept as a
//     sticky status readable through gbf_last_status();
//   * single domain only (size == 1, the no_communication path);
//   * split mode (gbf_dropin_set_mode(2)) is the fused mode in the headline
//     split form: the step runs on an FP32 state with FP64-precision masses
//     (GBF_PREC_SPLIT) kept beside the caller's arrays, formed anew from the
//     caller's P1 and S2 whenever the host wrote them; P1 and S2 are written
//     back, and the derived arrays formed as in the fused mode from the state
//     the step started from, when the host reads them. Its results are the
//     split form's (max|dS| <= 1e-5, rel-L2(P) <= 1e-6 against the reference
//     arithmetic), not the reference's to round-off;
//   * fused mode (gbf_dropin_set_mode(1)) runs time_step_function's five
//     calls as one fused step that writes P1, S2, ro1, ro2 only; the other
//     arrays of the step (P2, Xi, velocities, roS, roS_old) are computed when
//     the host reads one of them, from the state the step started from, with
//     the same kernels as the one-call-per-stage mode. Its Newton stops once
//     an iteration moves S by less than 1e-11 and P by less than 1e-11 P
//     (at most the reference's 7 iterations): the same results to round-off
//     (the tests hold both modes to the oracle at 1e-12) in about a third of
//     the time, since every FP64 iteration costs a log and an exp per cell.
#include <stdio.h>
#include <stdlib.h>

#include <mutex>
#include <unordered_map>

#include "../../include/gbflow_dropin.h"
#include "gbf_internal.h"
#include "gbf_domain.h"

namespace {

// Hidden per-domain state, keyed by the device P1 pointer the caller holds.
struct DropinDomain {
  size_t alloc_cells = 0;
  double* boundary_scratch = nullptr;
  gbf_domain* fused = nullptr;  // created on first use in fused mode
};

std::mutex g_mu;
std::unordered_map<const double*, DropinDomain> g_domains;
// The mode a process starts in: GBF_DROPIN_MODE=1 (fused) or 2 (split) in the
// environment, for drivers that cannot call gbf_dropin_set_mode (the
// reference's own main.cpp); anything else, or nothing, the eager mode.
int initial_mode() {
  const char* e = getenv("GBF_DROPIN_MODE");
  if (!e || e[0] == '\0' || e[1] != '\0') return 0;
  return e[0] == '1' ? 1 : e[0] == '2' ? 2 : 0;
}
int g_mode = initial_mode();
constexpr double kFusedNewtonTol = 1e-11;  // converge-and-exit Newton of the fused mode

gbf_model model_from(const consts& def, int localNx) {
  gbf_model m;
  gbf_model_reference(&m, localNx, def.Ny, def.Nz, def.dt);
  if (g_mode != 0) m.newton_tol = kFusedNewtonTol;
  for (int md = 0; md < 2; md++) {
    m.K[md] = def.K[md];
    m.lambda[md] = def.lambda[md];
    m.S_wr[md] = def.S_wr[md];
    m.m[md] = def.m[md];
    m.P_d[md] = def.P_d[md];
  }
  m.h1 = def.h1; m.h2 = def.h2; m.h3 = def.h3;
  m.beta1 = def.beta1; m.beta2 = def.beta2;
  m.source = def.source;
  return m;
}

gbf_arrays arrays_from(const ptr_Arrays& D) {
  gbf_arrays a;
  a.P1 = D.P1; a.P2 = D.P2; a.S2 = D.S2; a.ro1 = D.ro1; a.ro2 = D.ro2;
  a.u1x = D.u1x; a.u1y = D.u1y; a.u1z = D.u1z; a.u2x = D.u2x; a.u2y = D.u2y; a.u2z = D.u2z;
  a.Xi1 = D.Xi1; a.Xi2 = D.Xi2; a.roS1 = D.roS1; a.roS1_old = D.roS1_old; a.roS2 = D.roS2; a.roS2_old = D.roS2_old;
  return a;
}

gbf_cells cells_from(const ptr_Arrays& D) {
  gbf_cells c;
  c.media = D.media;
  c.K = nullptr;
  c.phi = nullptr;
  return c;
}

bool single_domain(int size, const char* where) {
  if (size == 1) return true;
  static bool warned = false;
  if (!warned) {
    printf("gbflow: %s: only the single-domain (no_communication) path is supported, size=%d\n", where, size);
    warned = true;
  }
  gbf_fail(GBF_ERR_ARG, where);
  return false;
}

DropinDomain* find_domain(const double* P1) {
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_domains.find(P1);
  return it == g_domains.end() ? nullptr : &it->second;
}

gbf_domain* fused_of(const ptr_Arrays& D, const gbf_model& m) {
  DropinDomain* dd = find_domain(D.P1);
  if (!dd) {
    gbf_fail(GBF_ERR_STATE, "fused and split modes need arrays from device_memory_alloc");
    return nullptr;
  }
  if (!dd->fused) {
    const int precision = g_mode == 2 ? GBF_PREC_SPLIT : GBF_PREC_F64;
    if (gbf_domain_attach_dropin(&m, arrays_from(D), cells_from(D), precision, &dd->fused) != GBF_OK) return nullptr;
  }
  return dd->fused;
}

// Any host access observes completed stages: run what is deferred, bring the
// caller's P1 and S2 up to the split state when `dev` is one of them, and
// materialise the derived arrays of a fused step when `dev` is one of those.
void flush_all(const double* dev = nullptr) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_domains)
    if (gbf_domain* f = kv.second.fused) {
      gbf_dropin_flush(f);
      if (dev && (dev == f->caller.P1 || dev == f->caller.S2)) gbf_dropin_writeback(f);
      if (dev && gbf_dropin_is_derived(f, dev)) gbf_dropin_materialize(f);
    }
}

// The host writes `dev`: the caller's arrays current first (the host may
// overwrite one of P1, S2 and keep the other), then the note of the write.
void before_host_write(const double* dev) {
  flush_all(dev);
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_domains)
    if (gbf_domain* f = kv.second.fused) gbf_dropin_writeback(f);
}
void after_host_write(const double* dev) {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_domains)
    if (gbf_domain* f = kv.second.fused) gbf_dropin_host_wrote(f, dev);
}

// Every caller array current, and the fused or split domains released (a mode
// change; they are created again on first use in the new mode).
void settle_all() {
  std::lock_guard<std::mutex> lk(g_mu);
  for (auto& kv : g_domains)
    if (gbf_domain* f = kv.second.fused) {
      gbf_dropin_flush(f);
      gbf_dropin_materialize(f);
      gbf_dropin_writeback(f);
      gbf_domain_detach_dropin(f);
      kv.second.fused = nullptr;
    }
}

}  // namespace

// ---------------------------------------------------------------- hot path

void ro_P2_Xi_calculation(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, consts def, int localNx, int rank,
                          int size, int blocksX, int blocksY, int blocksZ) {
  (void)HostArraysPtr; (void)rank; (void)blocksX; (void)blocksY; (void)blocksZ;
  if (!single_domain(size, "ro_P2_Xi_calculation")) return;
  gbf_model m = model_from(def, localNx);
  if (g_mode != 0) {
    if (gbf_domain* f = fused_of(DevArraysPtr, m)) gbf_dropin_defer(f, m, 1);
    return;
  }
  gbf_props_f64(&m, arrays_from(DevArraysPtr), cells_from(DevArraysPtr), nullptr);
}

void u_calculation(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, int localNx, int rank, int size, int blocksX,
                   int blocksY, int blocksZ, consts def) {
  (void)HostArraysPtr; (void)rank; (void)blocksX; (void)blocksY; (void)blocksZ;
  if (!single_domain(size, "u_calculation")) return;
  gbf_model m = model_from(def, localNx);
  if (g_mode != 0) {
    if (gbf_domain* f = fused_of(DevArraysPtr, m)) gbf_dropin_defer(f, m, 2);
    return;
  }
  gbf_velocity_f64(&m, arrays_from(DevArraysPtr), nullptr);
}

void roS_calculation(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, consts def, double t, int localNx, int rank,
                     int size, int blocksX, int blocksY, int blocksZ) {
  (void)HostArraysPtr; (void)t; (void)rank; (void)blocksX; (void)blocksY; (void)blocksZ;
  if (!single_domain(size, "roS_calculation")) return;
  gbf_model m = model_from(def, localNx);
  if (g_mode != 0) {
    if (gbf_domain* f = fused_of(DevArraysPtr, m)) gbf_dropin_defer(f, m, 3);
    return;
  }
  gbf_mass_f64(&m, arrays_from(DevArraysPtr), cells_from(DevArraysPtr), nullptr);
}

void P1_S2_calculation(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, consts def, int localNx, int rank, int size,
                       int blocksX, int blocksY, int blocksZ) {
  (void)HostArraysPtr; (void)rank; (void)blocksX; (void)blocksY; (void)blocksZ;
  if (!single_domain(size, "P1_S2_calculation")) return;
  gbf_model m = model_from(def, localNx);
  if (g_mode != 0) {
    if (gbf_domain* f = fused_of(DevArraysPtr, m)) gbf_dropin_defer(f, m, 4);
    return;
  }
  gbf_newton_f64(&m, arrays_from(DevArraysPtr), cells_from(DevArraysPtr), nullptr);
}

void boundary_conditions(ptr_Arrays HostArraysPtr, ptr_Arrays DevArraysPtr, int localNx, int rank, int size,
                         int blocksX, int blocksY, int blocksZ, consts def) {
  (void)HostArraysPtr; (void)rank; (void)blocksX; (void)blocksY; (void)blocksZ;
  if (!single_domain(size, "boundary_conditions")) return;
  gbf_model m = model_from(def, localNx);
  if (g_mode != 0) {
    if (gbf_domain* f = fused_of(DevArraysPtr, m)) gbf_dropin_defer(f, m, 5);
    return;
  }
  DropinDomain* dd = find_domain(DevArraysPtr.P1);
  double* scratch = dd ? dd->boundary_scratch : nullptr;
  bool own = false;
  if (!scratch) {  // arrays not allocated by device_memory_alloc: temporary scratch
    if (gbf_cuda_check(cudaMalloc(&scratch, gbf_boundary_scratch_doubles(&m) * sizeof(double)), "boundary scratch")) return;
    own = true;
  }
  gbf_boundary_f64(&m, arrays_from(DevArraysPtr), scratch, nullptr);
  if (own) cudaFree(scratch);
}

// ------------------------------------------------------------ data movement

void load_data_to_host(double* HostArrayPtr, double* DevArrayPtr, int localNx, consts def) {
  size_t n = (size_t)localNx * def.Ny * def.Nz;
  if (g_mode != 0) flush_all(DevArrayPtr);
  gbf_cuda_check(cudaMemcpy(HostArrayPtr, DevArrayPtr, n * sizeof(double), cudaMemcpyDeviceToHost), "copy data to host");
}

void load_data_to_device(double* HostArrayPtr, double* DevArrayPtr, int localNx, consts def) {
  size_t n = (size_t)localNx * def.Ny * def.Nz;
  if (g_mode != 0) before_host_write(DevArrayPtr);  // the other derived arrays keep their values
  gbf_cuda_check(cudaMemcpy(DevArrayPtr, HostArrayPtr, n * sizeof(double), cudaMemcpyHostToDevice), "copy double data to device");
  if (g_mode != 0) after_host_write(DevArrayPtr);
}

void load_data_to_device_int(int* HostArrayPtr, int* DevArrayPtr, int localNx, consts def) {
  size_t n = (size_t)localNx * def.Ny * def.Nz;
  if (g_mode != 0) flush_all();  // deferred stages read the media array
  gbf_cuda_check(cudaMemcpy(DevArrayPtr, HostArrayPtr, n * sizeof(int), cudaMemcpyHostToDevice), "copy int data to device");
  if (g_mode != 0) {
    std::lock_guard<std::mutex> lk(g_mu);
    for (auto& kv : g_domains)
      if (gbf_domain* f = kv.second.fused) gbf_dropin_media_wrote(f, DevArrayPtr);
  }
}

void device_memory_alloc(ptr_Arrays* A, double** DevBuffer, int nX, consts def) {
  const size_t n = (size_t)nX * def.Ny * def.Nz;
  double** fields[] = {&A->x, &A->y, &A->z, &A->P1, &A->P2, &A->S2, &A->ro1, &A->ro2, &A->u1x, &A->u1y, &A->u1z,
                       &A->u2x, &A->u2y, &A->u2z, &A->Xi1, &A->Xi2, &A->roS1, &A->roS1_old, &A->roS2, &A->roS2_old};
  if (gbf_cuda_check(cudaMalloc((void**)DevBuffer, 2 * (size_t)def.Ny * def.Nz * sizeof(double)), "memory allocation")) return;
  for (double** f : fields)
    if (gbf_cuda_check(cudaMalloc((void**)f, n * sizeof(double)), "memory allocation")) return;
  if (gbf_cuda_check(cudaMalloc((void**)&A->media, n * sizeof(int)), "memory allocation")) return;
  // Zero everything: the reference leaves roS_old and the derived arrays
  // undefined until the first step writes them.
  for (double** f : fields) cudaMemset(*f, 0, n * sizeof(double));
  cudaMemset(A->media, 0, n * sizeof(int));
  DropinDomain dd;
  dd.alloc_cells = n;
  gbf_model m;
  gbf_model_reference(&m, nX, def.Ny, def.Nz, def.dt);
  size_t ns = gbf_boundary_scratch_doubles(&m);  // nX >= NX: large enough for the indexing stride NX
  if (ns && gbf_cuda_check(cudaMalloc(&dd.boundary_scratch, ns * sizeof(double)), "memory allocation")) return;
  std::lock_guard<std::mutex> lk(g_mu);
  g_domains[A->P1] = dd;
}

void device_memory_free(ptr_Arrays D, double* DevBuffer) {
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_domains.find(D.P1);
    if (it != g_domains.end()) {
      if (it->second.boundary_scratch) cudaFree(it->second.boundary_scratch);
      if (it->second.fused) gbf_domain_detach_dropin(it->second.fused);
      g_domains.erase(it);
    }
  }
  double* fields[] = {DevBuffer, D.x, D.y, D.z, D.P1, D.P2, D.S2, D.ro1, D.ro2, D.u1x, D.u1y, D.u1z,
                      D.u2x, D.u2y, D.u2z, D.Xi1, D.Xi2, D.roS1, D.roS1_old, D.roS2, D.roS2_old};
  for (double* f : fields) cudaFree(f);
  cudaFree(D.media);
  gbf_cuda_check(cudaGetLastError(), "memory release");
}

void Device_Initialize(int rank, int* blocksX, int* blocksY, int* blocksZ, int localNx, consts def) {
  int count = 0;
  if (gbf_cuda_check(cudaGetDeviceCount(&count), "cudaGetDeviceCount") || count < 1) return;
  int device = rank % count;
  if (gbf_cuda_check(cudaSetDevice(device), "cudaSetDevice")) return;
  printf("CUDA initialized.\n");
  // Block counts of the reference's 16x4x4 launch shape (gpu.cu:575-583);
  // main.cpp passes them back in, the kernels here size their own grids.
  *blocksX = (localNx + 15) / 16;
  *blocksY = (def.Ny + 3) / 4;
  *blocksZ = (def.Nz + 3) / 4;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) == cudaSuccess) {
    printf("Device %d\nCompute capability : %d.%d\nName : %s\nTotal Global Memory : %zu\n\n", device, p.major,
           p.minor, p.name, p.totalGlobalMem);
    size_t need = (size_t)(localNx + 3) * def.Ny * def.Nz * (21 * sizeof(double));
    if (need > p.totalGlobalMem) printf("\nError! Not enough memory at GPU, rank=%d\n", rank);
  }
  gbf_model m = model_from(def, localNx);
  if (gbf_model_validate(&m, nullptr, 0) != GBF_OK) printf("gbflow: invalid model parameters (grid dims must be >= 3)\n");
}

// ------------------------------------------------- halo pack / unpack (MPI)

namespace {
__global__ void k_pack_halo(const double* a, double* buf, int localNx, int ny, int nz) {
  int n = ny * nz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    int j = t % ny, k = t / ny;
    size_t row = (size_t)localNx * j + (size_t)localNx * ny * k;
    buf[j + ny * k] = a[1 + row];
    buf[j + ny * k + n] = a[localNx - 2 + row];
  }
}
__global__ void k_unpack_halo(double* a, const double* buf, int localNx, int ny, int nz, int rank, int size) {
  int n = ny * nz;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    int j = t % ny, k = t / ny;
    size_t row = (size_t)localNx * j + (size_t)localNx * ny * k;
    if (rank != 0) a[row] = buf[j + ny * k];
    if (rank != size - 1) a[localNx - 1 + row] = buf[j + ny * k + n];
  }
}
}  // namespace

// gpu.cu:626-632: pack the i = 1 and i = localNx-2 planes, copy to the host.
void load_exchange_data(double* HostArrayPtr, double* DevArrayPtr, double* HostBuffer, double* DevBuffer, int localNx,
                        int blocksY, int blocksZ, int rank, int size, consts def) {
  (void)HostArrayPtr; (void)blocksY; (void)blocksZ; (void)rank; (void)size;
  int n = def.Ny * def.Nz;
  k_pack_halo<<<(n + 255) / 256, 256>>>(DevArrayPtr, DevBuffer, localNx, def.Ny, def.Nz);
  if (gbf_cuda_check(cudaGetLastError(), "load_exchange_data")) return;
  gbf_cuda_check(cudaMemcpy(HostBuffer, DevBuffer, 2 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost), "copy data to host");
}

// gpu.cu:648-654: copy the received planes to the device, unpack into i = 0 / i = localNx-1.
void save_exchange_data(double* HostArrayPtr, double* DevArrayPtr, double* HostBuffer, double* DevBuffer, int localNx,
                        int blocksY, int blocksZ, int rank, int size, consts def) {
  (void)HostArrayPtr; (void)blocksY; (void)blocksZ;
  int n = def.Ny * def.Nz;
  if (gbf_cuda_check(cudaMemcpy(DevBuffer, HostBuffer, 2 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice), "copy data to device")) return;
  k_unpack_halo<<<(n + 255) / 256, 256>>>(DevArrayPtr, DevBuffer, localNx, def.Ny, def.Nz, rank, size);
  gbf_cuda_check(cudaGetLastError(), "save_exchange_data");
}

extern "C" {
int gbf_dropin_set_mode(int mode) {
  if (mode != 0 && mode != 1 && mode != 2) return gbf_fail(GBF_ERR_ARG, "gbf_dropin_set_mode");
  if (mode != g_mode) settle_all();
  g_mode = mode;
  return GBF_OK;
}
int gbf_dropin_get_mode(void) { return g_mode; }
gbf_domain* gbf_dropin_domain(const double* dev_P1) {
  DropinDomain* dd = find_domain(dev_P1);
  return dd ? dd->fused : nullptr;
}
}
