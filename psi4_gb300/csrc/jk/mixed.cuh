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
// Memory pressure: drop the split copies of B and the factor / X workspaces (rebuilt on next
// use) but keep the incremental history, which is still valid for the same B.
void mixed_release(MixedState* m);
size_t mixed_query_memory(int nbf, int naux, int max_nocc);
// K for the lr-symmetric density C C^T (C padded, device), written to K (nbf x nbf, device).
// map_host: the tile map of L on the host (the split copy of B keeps only the 128 x 32 blocks
// that touch a stored tile).
// Records `ev_transform_done` between the half-transform and the contraction.
int mixed_build_K(MixedState* m, const double* B, const TileLayout& L, const int* map_host, int nbf, int nbf_pad,
                  int naux, const double* Cpad, int nocc, int nocc_pad, int mode, double* K, cudaEvent_t ev_transform_done,
                  cudaStream_t stream, std::string& err);

// K (nbf x nbf, device) = [K_prev +] sum_Q B_Q (U+ U+^T - U- U-^T) B_Q, U device (nbf x nu, ldu).
int mixed_k_factor(MixedState* m, const double* B, const TileLayout& L, const int* map_host, int nbf, int naux,
                   const double* U, int ldu, int npos, int nneg, int accumulate, double* K, cudaEvent_t ev_transform_done,
                   cudaStream_t s, std::string& err);
// Make K (device, nbf x nbf, FP64) the base of the next incremental build.
int mixed_set_base(MixedState* m, const double* K, int nbf, cudaStream_t s, std::string& err);
// error bits raised by the tensor-core kernels since the last call (0 = none); clears them
int mixed_error_flag(MixedState* m, cudaStream_t s);
// Failure test of the bounded waits: one thread waits on an mbarrier that nothing arrives on,
// gives up after limit_ns and raises the wait error bit (2) in this state's flag word.
int mixed_wait_probe(MixedState* m, unsigned long long limit_ns, cudaStream_t s, std::string& err);

}  // namespace gdfjk
