// mixed.cuh — split-precision (BF16 slices, FP32 accumulation) exchange path.
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "common.cuh"

namespace gdfjk {

struct MixedState;

MixedState* mixed_create();
void mixed_destroy(MixedState* m);
// B changed: drop the split copies and the incremental history.
void mixed_invalidate(MixedState* m);
size_t mixed_query_memory(int nbf, int naux, int max_nocc);
// K for the lr-symmetric density C C^T (C padded, device), written to K (nbf x nbf, device).
// Records `ev_transform_done` between the half-transform and the contraction.
int mixed_build_K(MixedState* m, const double* B, const TileLayout& L, int nbf, int nbf_pad, int naux,
                  const double* Cpad, int nocc, int nocc_pad, int mode, double* K, cudaEvent_t ev_transform_done,
                  cudaStream_t stream, std::string& err);

}  // namespace gdfjk
