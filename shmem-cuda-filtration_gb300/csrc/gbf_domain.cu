// gbf_domain.cu — the single-domain object of the C ABI (gbf_domain_*) and
// the drop-in's deferred (fused) mode.
#include <math.h>
#include <string.h>

#include <vector>

#include "gbf_domain.h"
#include "gbf_split.h"

GbfDerived gbf_derive(const gbf_model& m) {
  GbfDerived d;
  for (int md = 0; md < 2; md++) {
    const double lam = m.lambda[md], swr = m.S_wr[md];
    d.inv_1mswr[md] = 1.0 / (1.0 - swr);
    d.e1[md] = (2. + 3. * lam) / lam;
    d.e2[md] = (2. + lam) / lam;
    d.m_inv_lam[md] = -1. / lam;
    d.inv_lam_1mswr[md] = 1.0 / (lam * (1.0 - swr));
  }
  d.neg_inv_mu1 = -1.0 / m.mu1;
  d.neg_inv_mu2 = -1.0 / m.mu2;
  d.inv_h1 = 1.0 / m.h1;
  d.inv_h2 = 1.0 / m.h2;
  d.inv_h3 = 1.0 / m.h3;
  d.V = m.h1 * m.h2 * m.h3;
  d.src = (m.source_mode == GBF_SOURCE_RATE && m.rate_cells > 0)
              ? m.rate / (double)(m.rate_cells * m.rate_cells) / d.V
              : 0.0;
  return d;
}

int gbf_domain_alloc(gbf_domain* d, void** p, size_t bytes) {
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess) {
    *p = nullptr;
    return gbf_cuda_check(e, "gbf_domain_alloc");
  }
  d->owned.push_back(*p);
  return GBF_OK;
}

namespace {

int alloc_f64_work(gbf_domain* d) {
  const size_t n = gbf_geo(d->m).n, b = n * sizeof(double);
  int s = GBF_OK;
  s |= gbf_domain_alloc(d, (void**)&d->L1, b);
  s |= gbf_domain_alloc(d, (void**)&d->L2, b);
  s |= gbf_domain_alloc(d, (void**)&d->ro1, b);
  s |= gbf_domain_alloc(d, (void**)&d->ro2, b);
  s |= gbf_domain_alloc(d, (void**)&d->lnSe, b);
  return s ? GBF_ERR_NOMEM : GBF_OK;
}

int alloc_common(gbf_domain* d) {
  int s = gbf_domain_alloc(d, (void**)&d->status, sizeof(unsigned));
  if (s) return s;
  s = gbf_domain_alloc(d, (void**)&d->mass_partials, 2 * sizeof(double) * (size_t)(gbf_f64_flux_grid(d->m) + 1024));
  if (s) return s;
  GBF_CUDA(cudaMemsetAsync(d->status, 0, sizeof(unsigned), d->stream));
  return GBF_OK;
}

void free_all(gbf_domain* d) {
  gbf_timer_free(&d->timer);
  for (cudaEvent_t e : d->pipe_ev) cudaEventDestroy(e);
  d->pipe_ev.clear();
  if (d->pipe_in) cudaStreamDestroy(d->pipe_in);
  if (d->pipe_out) cudaStreamDestroy(d->pipe_out);
  d->pipe_in = d->pipe_out = nullptr;
  for (void* p : d->owned) cudaFree(p);
  d->owned.clear();
  if (d->own_stream && d->stream) cudaStreamDestroy(d->stream);
  d->stream = nullptr;
}

// One FP64 step: current buffer -> next buffer, then flip. In drop-in mode
// the caller's arrays (buffer 0) always hold the latest state: the state the
// step starts from is first copied to buffer 1, where it stays for the lazily
// materialised derived arrays (gbf_dropin_materialize).
int f64_step(gbf_domain* d, int props_flags) {
  const int nxt = d->cur ^ 1;
  GbfF64Step s = {};
  if (d->borrowed) {
    const size_t b = gbf_geo(d->m).n * sizeof(double);
    GBF_CUDA(cudaMemcpyAsync(d->P[1], d->P[0], b, cudaMemcpyDeviceToDevice, d->stream));
    GBF_CUDA(cudaMemcpyAsync(d->S[1], d->S[0], b, cudaMemcpyDeviceToDevice, d->stream));
    s.P = d->P[1];
    s.S = d->S[1];
    s.Pn = d->P[0];
    s.Sn = d->S[0];
  } else {
    s.P = d->P[d->cur];
    s.S = d->S[d->cur];
    s.Pn = d->P[nxt];
    s.Sn = d->S[nxt];
  }
  s.L1 = d->L1; s.L2 = d->L2; s.ro1 = d->ro1; s.ro2 = d->ro2; s.lnSe = d->lnSe;
  s.Xi1 = d->outs.Xi1; s.Xi2 = d->outs.Xi2; s.P2 = d->outs.P2;
  s.u1x = d->outs.u1x; s.u1y = d->outs.u1y; s.u1z = d->outs.u1z;
  s.u2x = d->outs.u2x; s.u2y = d->outs.u2y; s.u2z = d->outs.u2z;
  if (d->outs.roS1) {
    s.roS1 = d->outs.roS1; s.roS2 = d->outs.roS2; s.roS1_old = d->outs.roS1_old; s.roS2_old = d->outs.roS2_old;
  }
  s.status = d->status;
  double* mass_out = nullptr;
  if ((d->out_flags & GBF_OUT_MASS) && d->mass_hist && d->mass_count < d->mass_cap) {
    s.mass_partials = d->mass_partials;
    mass_out = d->mass_hist + 2 * d->mass_count;
    d->mass_count++;
  }
  if (d->borrowed) {  // the reference's own ro1/ro2 arrays hold the densities
    s.ro1 = d->caller.ro1;
    s.ro2 = d->caller.ro2;
  }
  int st = gbf_f64_launch_step(d->m, d->d, d->cells, s, props_flags, mass_out, d->stream, &d->timer);
  if (st) return st;
  if (d->borrowed)
    d->lazy_dirty = true;
  else
    d->cur = nxt;
  d->steps++;
  return GBF_OK;
}

int copy_cells(gbf_domain* d, const gbf_cells* hc) {
  const size_t n = gbf_geo(d->m).n;
  if (!hc) return GBF_OK;
  if (hc->media) {
    if (int s = gbf_domain_alloc(d, (void**)&d->own_media, n * sizeof(int))) return s;
    GBF_CUDA(cudaMemcpy(d->own_media, hc->media, n * sizeof(int), cudaMemcpyHostToDevice));
    d->cells.media = d->own_media;
  }
  if (hc->K) {
    if (int s = gbf_domain_alloc(d, (void**)&d->own_K, n * sizeof(float))) return s;
    GBF_CUDA(cudaMemcpy(d->own_K, hc->K, n * sizeof(float), cudaMemcpyHostToDevice));
    d->cells.K = d->own_K;
  }
  if (hc->phi) {
    if (int s = gbf_domain_alloc(d, (void**)&d->own_phi, n * sizeof(float))) return s;
    GBF_CUDA(cudaMemcpy(d->own_phi, hc->phi, n * sizeof(float), cudaMemcpyHostToDevice));
    d->cells.phi = d->own_phi;
  }
  return GBF_OK;
}

}  // namespace

extern "C" {

int gbf_domain_create(const gbf_model* m, const gbf_cells* host_cells, int precision, gbf_domain** out) {
  if (!out) return gbf_fail(GBF_ERR_ARG, "gbf_domain_create: out");
  *out = nullptr;
  if (int s = gbf_model_validate(m, host_cells, 0)) return s;
  if (precision != GBF_PREC_F64 && precision != GBF_PREC_SPLIT && precision != GBF_PREC_SPLIT_DF &&
      precision != GBF_PREC_SPLIT_DEFECT)
    return gbf_fail(GBF_ERR_ARG, "precision");
  gbf_domain* d = new gbf_domain();
  d->m = *m;
  d->d = gbf_derive(*m);
  d->precision = precision;
  int s = GBF_OK;
  if (cudaStreamCreateWithFlags(&d->stream, cudaStreamNonBlocking) != cudaSuccess) s = gbf_fail(GBF_ERR_CUDA, "stream");
  d->own_stream = true;
  const size_t n = gbf_geo(*m).n;
  if (!s) s = copy_cells(d, host_cells);
  if (!s) s = alloc_common(d);
  if (!s && precision == GBF_PREC_F64) {
    for (int b = 0; b < 2 && !s; b++) {
      s |= gbf_domain_alloc(d, (void**)&d->P[b], n * sizeof(double));
      s |= gbf_domain_alloc(d, (void**)&d->S[b], n * sizeof(double));
    }
    if (!s) s = alloc_f64_work(d);
  }
  if (!s && precision != GBF_PREC_F64) s = gbf_split_alloc(d);
  if (s) {
    free_all(d);
    delete d;
    return gbf_fail(s, "gbf_domain_create");
  }
  *out = d;
  return GBF_OK;
}

int gbf_domain_destroy(gbf_domain* d) {
  if (!d) return GBF_OK;
  if (d->stream) cudaStreamSynchronize(d->stream);
  free_all(d);
  delete d;
  return GBF_OK;
}

int gbf_domain_set_stream(gbf_domain* d, void* stream) {
  if (!d) return gbf_fail(GBF_ERR_ARG, "gbf_domain_set_stream");
  GBF_CUDA(cudaStreamSynchronize(d->stream));
  if (d->own_stream) cudaStreamDestroy(d->stream);
  d->stream = (cudaStream_t)stream;
  d->own_stream = false;
  return GBF_OK;
}

int gbf_domain_set_outputs(gbf_domain* d, int flags, int mass_cap) {
  if (!d || mass_cap < 0) return gbf_fail(GBF_ERR_ARG, "gbf_domain_set_outputs");
  if (d->precision != GBF_PREC_F64 && (flags & (GBF_OUT_VELOCITY | GBF_OUT_MASS_ARRAYS)))
    return gbf_fail(GBF_ERR_ARG, "velocity/mass arrays are FP64-only outputs");
  const size_t n = gbf_geo(d->m).n, b = n * sizeof(double);
  if ((flags & GBF_OUT_MASS) && mass_cap > d->mass_cap) {
    if (int s = gbf_domain_alloc(d, (void**)&d->mass_hist, 2 * sizeof(double) * (size_t)mass_cap)) return s;
    if (int s = gbf_domain_alloc(d, (void**)&d->cfl_hist, 2 * sizeof(float) * (size_t)mass_cap)) return s;
    d->mass_cap = mass_cap;
    d->mass_count = 0;
  }
  if (d->cfl_hist) GBF_CUDA(cudaMemsetAsync(d->cfl_hist, 0, 2 * sizeof(float) * (size_t)d->mass_cap, d->stream));
  if ((flags & GBF_OUT_VELOCITY) && !d->outs.u1x) {
    double** f[] = {&d->outs.u1x, &d->outs.u1y, &d->outs.u1z, &d->outs.u2x, &d->outs.u2y, &d->outs.u2z};
    for (double** p : f)
      if (int s = gbf_domain_alloc(d, (void**)p, b)) return s;
  }
  if ((flags & GBF_OUT_MASS_ARRAYS) && !d->outs.roS1) {
    double** f[] = {&d->outs.roS1, &d->outs.roS2, &d->outs.roS1_old, &d->outs.roS2_old};
    for (double** p : f)
      if (int s = gbf_domain_alloc(d, (void**)p, b)) return s;
  }
  if ((flags & GBF_OUT_PROPS) && !d->outs.Xi1 && d->precision == GBF_PREC_F64) {
    double** f[] = {&d->outs.Xi1, &d->outs.Xi2, &d->outs.P2};
    for (double** p : f)
      if (int s = gbf_domain_alloc(d, (void**)p, b)) return s;
  }
  d->out_flags = flags;
  return GBF_OK;
}

int gbf_domain_upload_device(gbf_domain* d, const double* P1, const double* S2) {
  if (!d || !P1 || !S2) return gbf_fail(GBF_ERR_ARG, "gbf_domain_upload_device");
  const size_t b = gbf_geo(d->m).n * sizeof(double);
  if (d->precision != GBF_PREC_F64) {
    if (int s = gbf_split_upload(d, P1, S2, cudaMemcpyDeviceToDevice)) return s;
  } else {
    d->cur = 0;
    GBF_CUDA(cudaMemcpyAsync(d->P[0], P1, b, cudaMemcpyDeviceToDevice, d->stream));
    GBF_CUDA(cudaMemcpyAsync(d->S[0], S2, b, cudaMemcpyDeviceToDevice, d->stream));
  }
  d->mass_count = 0;
  d->steps = 0;
  d->uploaded = true;
  if (d->cfl_hist) GBF_CUDA(cudaMemsetAsync(d->cfl_hist, 0, 2 * sizeof(float) * (size_t)d->mass_cap, d->stream));
  GBF_CUDA(cudaMemsetAsync(d->status, 0, sizeof(unsigned), d->stream));
  return GBF_OK;
}

int gbf_domain_upload(gbf_domain* d, const double* P1, const double* S2) {
  if (!d || !P1 || !S2) return gbf_fail(GBF_ERR_ARG, "gbf_domain_upload");
  const size_t b = gbf_geo(d->m).n * sizeof(double);
  if (d->precision != GBF_PREC_F64) {
    if (int s = gbf_split_upload(d, P1, S2, cudaMemcpyHostToDevice)) return s;
  } else {
    d->cur = 0;
    GBF_CUDA(cudaMemcpyAsync(d->P[0], P1, b, cudaMemcpyHostToDevice, d->stream));
    GBF_CUDA(cudaMemcpyAsync(d->S[0], S2, b, cudaMemcpyHostToDevice, d->stream));
  }
  d->mass_count = 0;
  d->steps = 0;
  d->uploaded = true;
  if (d->cfl_hist) GBF_CUDA(cudaMemsetAsync(d->cfl_hist, 0, 2 * sizeof(float) * (size_t)d->mass_cap, d->stream));
  GBF_CUDA(cudaMemsetAsync(d->status, 0, sizeof(unsigned), d->stream));
  return GBF_OK;
}

int gbf_domain_advance_host(gbf_domain* d, const double* P_in, const double* S_in, int nsteps, double* P_out,
                            double* S_out) {
  if (!d || !P_in || !S_in || !P_out || !S_out || nsteps < 0) return gbf_fail(GBF_ERR_ARG, "gbf_domain_advance_host");
  if (d->borrowed) return gbf_fail(GBF_ERR_STATE, "gbf_domain_advance_host on a drop-in domain");
  if (d->precision != GBF_PREC_F64 && nsteps == 1 && !d->split_patch && gbf_split_pipelined(d->m))
    return gbf_split_advance_host(d, P_in, S_in, P_out, S_out);
  if (int s = gbf_domain_upload(d, P_in, S_in)) return s;
  if (int s = gbf_domain_step(d, nsteps)) return s;
  if (int s = gbf_domain_download(d, GBF_FIELD_P1, P_out)) return s;
  return gbf_domain_download(d, GBF_FIELD_S2, S_out);
}

int gbf_domain_step(gbf_domain* d, int nsteps) {
  if (!d || nsteps < 0) return gbf_fail(GBF_ERR_ARG, "gbf_domain_step");
  if (!d->uploaded) return gbf_fail(GBF_ERR_STATE, "gbf_domain_step before upload");
  int pf = 0;
  if (d->outs.Xi1) pf |= GBF_PF_WRITE_XI_P2;
  if (d->outs.u1x && (d->out_flags & GBF_OUT_VELOCITY)) pf |= GBF_PF_WRITE_U;
  for (int s = 0; s < nsteps; s++) {
    int st = (d->precision != GBF_PREC_F64) ? gbf_split_step(d) : f64_step(d, pf);
    if (st) return st;
  }
  return GBF_OK;
}

int gbf_domain_launches_per_step(gbf_domain* d) {
  if (!d) return 0;
  if (d->precision != GBF_PREC_F64) return gbf_split_launches_per_step(d);
  return 3 + ((d->out_flags & GBF_OUT_MASS) ? 1 : 0);
}

int gbf_domain_sync(gbf_domain* d) {
  if (!d) return gbf_fail(GBF_ERR_ARG, "gbf_domain_sync");
  GBF_CUDA(cudaStreamSynchronize(d->stream));
  return GBF_OK;
}

int gbf_domain_status(gbf_domain* d) {
  if (!d) return gbf_fail(GBF_ERR_ARG, "gbf_domain_status");
  unsigned h = 0;
  GBF_CUDA(cudaMemcpyAsync(&h, d->status, sizeof(unsigned), cudaMemcpyDeviceToHost, d->stream));
  GBF_CUDA(cudaStreamSynchronize(d->stream));
  if (h & GBF_DEV_TIMEOUT) return gbf_fail(GBF_ERR_TIMEOUT, "device wait timed out");
  if (h & GBF_DEV_NONFINITE) return gbf_fail(GBF_ERR_NONFINITE, "non-finite P or S");
  return GBF_OK;
}

long long gbf_domain_steps_done(gbf_domain* d) { return d ? d->steps : -1; }

// Checkpoint in the reference's save/save.dat layout (gbf_checkpoint.cpp).
// roS1_old, roS2_old are what the reference holds after its last step: the
// start-of-step masses of the interior cells, i.e. of the state before that
// step, which is still in the other ping-pong buffer (zeros before a step).
int gbf_domain_save(gbf_domain* d, const char* path, int step) {
  if (!d || !path) return gbf_fail(GBF_ERR_ARG, "gbf_domain_save");
  if (!d->uploaded || d->borrowed) return gbf_fail(GBF_ERR_STATE, "gbf_domain_save without an uploaded state");
  const size_t n = gbf_geo(d->m).n;
  std::vector<double> P(n), S(n), old(2 * n, 0.0);
  std::vector<int> media;
  if (int s = gbf_domain_download(d, GBF_FIELD_P1, P.data())) return s;
  if (int s = gbf_domain_download(d, GBF_FIELD_S2, S.data())) return s;
  if (d->steps > 0) {
    double* tmp = nullptr;
    GBF_CUDA(cudaMallocAsync((void**)&tmp, 2 * n * sizeof(double), d->stream));
    const int prev = d->cur ^ 1;
    int s = d->precision == GBF_PREC_F64
                ? gbf_roS_old_launch(d->m, d->P[prev], d->S[prev], nullptr, nullptr, tmp, tmp + n, d->stream)
                : gbf_roS_old_launch(d->m, nullptr, nullptr, d->Pf[prev], d->Sf[prev], tmp, tmp + n, d->stream);
    if (!s) s = gbf_cuda_check(cudaMemcpyAsync(old.data(), tmp, 2 * n * sizeof(double), cudaMemcpyDeviceToHost,
                                               d->stream), "copy roS_old");
    cudaFreeAsync(tmp, d->stream);
    if (!s) s = gbf_cuda_check(cudaStreamSynchronize(d->stream), "gbf_domain_save");
    if (s) return s;
  }
  if (d->cells.media) {
    media.resize(n);
    GBF_CUDA(cudaMemcpy(media.data(), d->cells.media, n * sizeof(int), cudaMemcpyDeviceToHost));
  }
  return gbf_checkpoint_write(path, &d->m, step, P.data(), S.data(), old.data(), old.data() + n,
                              media.empty() ? nullptr : media.data());
}

// The reference's Tecplot files of the domain's state (gbf_plots.cpp). Like
// the reference's u arrays after a step, the velocities are those of the
// state the last step started from (a2 runs before a3-a5, main.cpp:85-92),
// computed with the one-call-per-stage kernels; zeros before the first step.
int gbf_domain_write_plots(gbf_domain* d, const char* dir, double t) {
  if (!d || !dir) return gbf_fail(GBF_ERR_ARG, "gbf_domain_write_plots");
  if (!d->uploaded || d->borrowed) return gbf_fail(GBF_ERR_STATE, "gbf_domain_write_plots without an uploaded state");
  const gbf_model& m = d->m;
  const size_t n = gbf_geo(m).n, b = n * sizeof(double);
  std::vector<double> P(n), S(n), u(3 * n, 0.0);
  std::vector<int> media;
  if (int s = gbf_domain_download(d, GBF_FIELD_P1, P.data())) return s;
  if (int s = gbf_domain_download(d, GBF_FIELD_S2, S.data())) return s;
  if (d->steps > 0) {
    double* w = nullptr;  // P1, S2, P2, ro1, ro2, Xi1, Xi2, u1x, u1y, u1z, u2x, u2y, u2z
    GBF_CUDA(cudaMallocAsync((void**)&w, 13 * b, d->stream));
    gbf_arrays a = {};
    a.P1 = w; a.S2 = w + n; a.P2 = w + 2 * n; a.ro1 = w + 3 * n; a.ro2 = w + 4 * n; a.Xi1 = w + 5 * n;
    a.Xi2 = w + 6 * n; a.u1x = w + 7 * n; a.u1y = w + 8 * n; a.u1z = w + 9 * n; a.u2x = w + 10 * n;
    a.u2y = w + 11 * n; a.u2z = w + 12 * n;
    const int prev = d->cur ^ 1;
    int s = d->precision == GBF_PREC_F64 ? gbf_cuda_check(cudaMemcpyAsync(a.P1, d->P[prev], b, cudaMemcpyDeviceToDevice, d->stream), "copy P")
                                         : gbf_split_state_to_f64(m, d->split_rows, d->Pf[prev], d->Sf[prev], a.P1, a.S2, d->stream);
    if (!s && d->precision == GBF_PREC_F64)
      s = gbf_cuda_check(cudaMemcpyAsync(a.S2, d->S[prev], b, cudaMemcpyDeviceToDevice, d->stream), "copy S");
    if (!s) s = gbf_props_f64(&m, a, d->cells, d->stream);
    if (!s) s = gbf_velocity_f64(&m, a, d->stream);
    if (!s) s = gbf_cuda_check(cudaMemcpyAsync(u.data(), a.u2x, 3 * b, cudaMemcpyDeviceToHost, d->stream), "copy u");
    cudaFreeAsync(w, d->stream);
    if (!s) s = gbf_cuda_check(cudaStreamSynchronize(d->stream), "gbf_domain_write_plots");
    if (s) return s;
  }
  if (d->cells.media) {
    media.resize(n);
    GBF_CUDA(cudaMemcpy(media.data(), d->cells.media, n * sizeof(int), cudaMemcpyDeviceToHost));
  }
  return gbf_write_plots(dir, &m, t, P.data(), S.data(), u.data(), u.data() + n, u.data() + 2 * n,
                         media.empty() ? nullptr : media.data());
}

// Restore (P1, S2) from such a file; its media must equal the domain's
// (all 0 for a domain without a media table).
int gbf_domain_restore(gbf_domain* d, const char* path, int* step) {
  if (!d || !path) return gbf_fail(GBF_ERR_ARG, "gbf_domain_restore");
  if (d->borrowed) return gbf_fail(GBF_ERR_STATE, "gbf_domain_restore on a drop-in domain");
  const size_t n = gbf_geo(d->m).n;
  std::vector<double> P(n), S(n);
  std::vector<int> media(n), mine(n, 0);
  int j = 0;
  if (int s = gbf_checkpoint_read(path, &d->m, &j, P.data(), S.data(), nullptr, nullptr, media.data())) return s;
  if (d->cells.media) GBF_CUDA(cudaMemcpy(mine.data(), d->cells.media, n * sizeof(int), cudaMemcpyDeviceToHost));
  if (media != mine) return gbf_fail(GBF_ERR_ARG, "gbf_domain_restore: the file's media differ from the domain's");
  if (int s = gbf_domain_upload(d, P.data(), S.data())) return s;
  if (step) *step = j;
  return GBF_OK;
}
int gbf_domain_uses_tma(gbf_domain* d) { return d && d->tma ? 1 : 0; }

int gbf_domain_set_timing(gbf_domain* d, int on) {
  if (!d) return gbf_fail(GBF_ERR_ARG, "gbf_domain_set_timing");
  d->timer.on = on != 0;
  return GBF_OK;
}

int gbf_domain_kernel_times(gbf_domain* d, double* ms, int* launches, int nkinds) {
  if (!d || !ms || !launches || nkinds < 0) return gbf_fail(GBF_ERR_ARG, "gbf_domain_kernel_times");
  return gbf_timer_collect(&d->timer, ms, launches, nkinds);
}

int gbf_domain_download(gbf_domain* d, int field, double* host) {
  if (!d || !host || field < 0 || field >= GBF_FIELD_COUNT) return gbf_fail(GBF_ERR_ARG, "gbf_domain_download");
  const size_t n = gbf_geo(d->m).n, b = n * sizeof(double);
  if (d->precision != GBF_PREC_F64) return gbf_split_download(d, field, host);
  const double* src = nullptr;
  switch (field) {
    case GBF_FIELD_P1: src = d->P[d->cur]; break;
    case GBF_FIELD_S2: src = d->S[d->cur]; break;
    case GBF_FIELD_RO1: src = d->ro1; break;
    case GBF_FIELD_RO2: src = d->ro2; break;
    case GBF_FIELD_P2: src = d->outs.P2; break;
    case GBF_FIELD_XI1: src = d->outs.Xi1; break;
    case GBF_FIELD_XI2: src = d->outs.Xi2; break;
    case GBF_FIELD_U1X: src = d->outs.u1x; break;
    case GBF_FIELD_U1Y: src = d->outs.u1y; break;
    case GBF_FIELD_U1Z: src = d->outs.u1z; break;
    case GBF_FIELD_U2X: src = d->outs.u2x; break;
    case GBF_FIELD_U2Y: src = d->outs.u2y; break;
    case GBF_FIELD_U2Z: src = d->outs.u2z; break;
    case GBF_FIELD_ROS1: src = d->outs.roS1; break;
    case GBF_FIELD_ROS2: src = d->outs.roS2; break;
    case GBF_FIELD_ROS1_OLD: src = d->outs.roS1_old; break;
    case GBF_FIELD_ROS2_OLD: src = d->outs.roS2_old; break;
  }
  if (!src) return gbf_fail(GBF_ERR_STATE, "field not produced (enable it with gbf_domain_set_outputs)");
  GBF_CUDA(cudaMemcpyAsync(host, src, b, cudaMemcpyDeviceToHost, d->stream));
  GBF_CUDA(cudaStreamSynchronize(d->stream));
  return GBF_OK;
}

int gbf_domain_cfl_history(gbf_domain* d, float* host, int max_steps, int* nsteps_out) {
  if (!d || !host || max_steps < 0) return gbf_fail(GBF_ERR_ARG, "gbf_domain_cfl_history");
  long long n = d->mass_count < max_steps ? d->mass_count : max_steps;
  if (n > 0 && d->cfl_hist)
    GBF_CUDA(cudaMemcpyAsync(host, d->cfl_hist, 2 * sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, d->stream));
  GBF_CUDA(cudaStreamSynchronize(d->stream));
  if (nsteps_out) *nsteps_out = (int)n;
  return GBF_OK;
}

int gbf_domain_mass_history(gbf_domain* d, double* host, int max_steps, int* nsteps_out) {
  if (!d || !host || max_steps < 0) return gbf_fail(GBF_ERR_ARG, "gbf_domain_mass_history");
  long long n = d->mass_count < max_steps ? d->mass_count : max_steps;
  if (n > 0) {
    GBF_CUDA(cudaMemcpyAsync(host, d->mass_hist, 2 * sizeof(double) * (size_t)n, cudaMemcpyDeviceToHost, d->stream));
  }
  GBF_CUDA(cudaStreamSynchronize(d->stream));
  if (nsteps_out) *nsteps_out = (int)n;
  return GBF_OK;
}

}  // extern "C"

// ------------------------------------------------------------------ drop-in

int gbf_domain_attach_dropin(const gbf_model* m, gbf_arrays caller, gbf_cells cells, int precision, gbf_domain** out) {
  *out = nullptr;
  if (int s = gbf_model_validate(m, nullptr, 0)) return s;
  gbf_domain* d = new gbf_domain();
  d->m = *m;
  d->d = gbf_derive(*m);
  d->precision = precision;
  d->borrowed = true;
  d->caller = caller;
  d->cells = cells;
  d->stream = nullptr;  // legacy default stream, as the reference's launches
  d->uploaded = true;
  const size_t n = gbf_geo(*m).n;
  int s = alloc_common(d);
  d->P[0] = caller.P1;
  d->S[0] = caller.S2;
  if (!s) s |= gbf_domain_alloc(d, (void**)&d->P[1], n * sizeof(double));
  if (!s) s |= gbf_domain_alloc(d, (void**)&d->S[1], n * sizeof(double));
  if (!s) s = precision == GBF_PREC_F64 ? alloc_f64_work(d) : gbf_split_alloc(d);
  if (!s) s = gbf_domain_alloc(d, (void**)&d->bscratch, gbf_boundary_scratch_doubles(m) * sizeof(double));
  if (s) {
    free_all(d);
    delete d;
    return s;
  }
  // The fused step writes P1, S2 (and the densities ro1, ro2); the other
  // arrays the reference's five calls write are materialised on demand.
  d->outs = {};
  d->out_flags = 0;
  *out = d;
  return GBF_OK;
}

// The derived arrays of the reference's step (a1: P2, Xi1, Xi2, ro1, ro2;
// a2: velocities; a3: roS1, roS2, roS1_old, roS2_old) after the last fused
// step: the eager stage kernels run on the state that step started from.
int gbf_dropin_materialize(gbf_domain* d) {
  if (!d || !d->lazy_dirty) return GBF_OK;
  gbf_arrays a = d->caller;
  a.P1 = d->P[1];
  a.S2 = d->S[1];
  if (d->precision != GBF_PREC_F64) {  // split mode: the step-start state is the other split buffer
    if (int s = gbf_split_state_to_f64(d->m, d->split_rows, d->Pf[d->cur ^ 1], d->Sf[d->cur ^ 1], d->P[1], d->S[1],
                                       d->stream))
      return s;
  }
  int s = gbf_props_f64(&d->m, a, d->cells, nullptr);
  s |= gbf_velocity_f64(&d->m, a, nullptr);
  s |= gbf_mass_f64(&d->m, a, d->cells, nullptr);
  d->lazy_dirty = false;
  return s;
}

bool gbf_dropin_is_derived(const gbf_domain* d, const double* p) {
  const gbf_arrays& c = d->caller;
  const double* derived[] = {c.P2, c.ro1, c.ro2, c.Xi1, c.Xi2, c.u1x, c.u1y, c.u1z,
                             c.u2x, c.u2y, c.u2z, c.roS1, c.roS2, c.roS1_old, c.roS2_old};
  for (const double* q : derived)
    if (q == p) return true;
  return false;
}

void gbf_domain_detach_dropin(gbf_domain* d) {
  if (!d) return;
  cudaDeviceSynchronize();
  free_all(d);
  delete d;
}

int gbf_dropin_writeback(gbf_domain* d) {
  if (!d || !d->caller_stale) return GBF_OK;
  d->caller_stale = false;
  return gbf_split_state_to_f64(d->m, d->split_rows, d->Pf[d->cur], d->Sf[d->cur], d->caller.P1, d->caller.S2,
                                d->stream);
}

void gbf_dropin_host_wrote(gbf_domain* d, const double* dev) {
  if (d && d->precision != GBF_PREC_F64 && (dev == d->caller.P1 || dev == d->caller.S2)) d->split_stale = true;
}

int gbf_dropin_media_wrote(gbf_domain* d, const int* dev) {
  if (!d || dev != d->cells.media || !gbf_is_defect(gbf_mass_rep(d->precision))) return GBF_OK;
  return gbf_defect_k1(d->m, d->cells.phi, d->cells.media, &d->defect_k1v, nullptr);
}

// Run the pending stages (bitmask of stages 1..4) one kernel each, in order.
int gbf_dropin_flush(gbf_domain* d) {
  if (!d || !d->pending) return GBF_OK;
  const gbf_arrays a = d->caller;
  // the arrays these stages do not rewrite keep the last fused step's values
  int s = gbf_dropin_materialize(d);
  s |= gbf_dropin_writeback(d);  // split mode: the stages run on the caller's P1, S2
  if (d->precision != GBF_PREC_F64 && (d->pending & 8)) d->split_stale = true;  // the Newton rewrites them
  if (d->pending & 1) s |= gbf_props_f64(&d->m, a, d->cells, nullptr);
  if (d->pending & 2) s |= gbf_velocity_f64(&d->m, a, nullptr);
  if (d->pending & 4) s |= gbf_mass_f64(&d->m, a, d->cells, nullptr);
  if (d->pending & 8) s |= gbf_newton_f64(&d->m, a, d->cells, nullptr);
  d->pending = 0;
  return s;
}

// Stage k (1..5) of time_step_function (main.cpp:86-92). Stages 1-4 are
// recorded; stage 5 runs the fused step when 1-4 came in order since the
// last step. Any other sequence falls back to one kernel per stage.
int gbf_dropin_defer(gbf_domain* d, const gbf_model& m, int stage) {
  if (memcmp(&m, &d->m, sizeof(gbf_model)) != 0) {  // parameters changed between calls
    // under the old parameters: the deferred stages, the last step's derived
    // arrays, and (split mode) the caller's P1, S2 from the split state, whose
    // dP and mass defects are taken against the old rows' hydrostatic values
    if (int s = gbf_dropin_flush(d)) return s;
    if (int s = gbf_dropin_materialize(d)) return s;
    if (int s = gbf_dropin_writeback(d)) return s;
    d->m = m;
    d->d = gbf_derive(m);
    if (d->precision != GBF_PREC_F64) {  // split mode: its row constants, and the state formed anew
      if (int s = gbf_split_fill_rows(d->m, d->split_rows, d->stream)) return s;
      d->split_stale = true;
      if (gbf_is_defect(gbf_mass_rep(d->precision)))
        if (int s = gbf_defect_k1(d->m, d->cells.phi, d->cells.media, &d->defect_k1v, nullptr)) return s;
    }
  }
  const int prefix = (1 << (stage - 1)) - 1;
  if (stage <= 4) {
    if (d->pending == prefix) {
      d->pending |= 1 << (stage - 1);
      return GBF_OK;
    }
    int s = gbf_dropin_flush(d);
    d->pending = 1 << (stage - 1);
    return s | gbf_dropin_flush(d);
  }
  if (d->pending == 15) {  // the whole step: fused (its derived arrays are left to materialise on demand)
    d->pending = 0;
    if (d->precision == GBF_PREC_F64) return f64_step(d, 0);
    // split mode: the split state from the caller's arrays when they were
    // written since, one split step (the caller's P1, S2 are written back
    // when read)
    if (d->split_stale) {
      if (int s = gbf_split_upload(d, d->caller.P1, d->caller.S2, cudaMemcpyDeviceToDevice)) return s;
      d->split_stale = false;
    }
    if (int s = gbf_split_step(d)) return s;
    d->caller_stale = true;
    d->lazy_dirty = true;
    return GBF_OK;
  }
  int s = gbf_dropin_flush(d);
  if (!s) s = gbf_dropin_materialize(d);
  if (!s) s = gbf_dropin_writeback(d);
  if (d->precision != GBF_PREC_F64) d->split_stale = true;  // the boundary rules rewrite P1, S2
  return s | gbf_boundary_f64(&d->m, d->caller, d->bscratch, nullptr);
}
