// gbf_split.cu — split-precision step (FP32 P, S, K, fluxes; FP64 masses).
#include "gbf_split.h"

int gbf_split_alloc(gbf_domain* d) { (void)d; return gbf_fail(GBF_ERR_ARG, "split precision not built yet"); }
int gbf_split_upload(gbf_domain* d, const double* P1, const double* S2, cudaMemcpyKind kind) {
  (void)d; (void)P1; (void)S2; (void)kind;
  return gbf_fail(GBF_ERR_ARG, "split precision not built yet");
}
int gbf_split_step(gbf_domain* d) { (void)d; return gbf_fail(GBF_ERR_ARG, "split precision not built yet"); }
int gbf_split_download(gbf_domain* d, int field, double* host) {
  (void)d; (void)field; (void)host;
  return gbf_fail(GBF_ERR_ARG, "split precision not built yet");
}
int gbf_split_launches_per_step(gbf_domain* d) { (void)d; return 0; }
