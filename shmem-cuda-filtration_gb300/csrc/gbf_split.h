// gbf_split.h — split-precision (FP32 state, FP64 masses) domain launchers.
#pragma once

#include "gbf_domain.h"

int gbf_split_alloc(gbf_domain* d);
int gbf_split_upload(gbf_domain* d, const double* P1, const double* S2, cudaMemcpyKind kind);
int gbf_split_step(gbf_domain* d);
int gbf_split_download(gbf_domain* d, int field, double* host);
int gbf_split_launches_per_step(gbf_domain* d);
