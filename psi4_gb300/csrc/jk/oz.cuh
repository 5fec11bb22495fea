// oz.cuh — FP64-accurate exchange on the BF16 tensor cores (Ozaki-style digit splitting).
#pragma once
#include <cuda_runtime.h>

#include <string>

#include "common.cuh"

namespace gdfjk {

struct OzState;

OzState* oz_create();
void oz_destroy(OzState* o);
// B changed: drop the digit copy of B.
void oz_invalidate(OzState* o);
// Release the digit copy of B and the X buffers (another form needs the memory).
void oz_release(OzState* o);
size_t oz_query_memory(int nbf, int naux, int max_nocc);
// K (nbf x nbf, device) = sum_Q (B_Q C_left)(B_Q C_right)^T (C device, nbf_pad x nocc_pad,
// row-major; Crpad = nullptr for the lr-symmetric C C^T); records `ev_transform_done` after
// the last half-transform.  map_host: the tile map of L on the host (digits of B are kept
// only where a stored tile is).  With o_right, the right factor uses a second tensor
// (B_right, same tile map, its digits kept on o_right): sum_Q (B_Q C_left)(B'_Q C_right)^T.
int oz_build_K(OzState* o, const double* B, const TileLayout& L, const int* map_host, int nbf, int naux, const double* Cpad,
               const double* Crpad, int nocc, int nocc_pad, double* K, cudaEvent_t ev_transform_done, cudaStream_t s,
               std::string& err, OzState* o_right = nullptr, const double* B_right = nullptr,
               const TileLayout* L_right = nullptr);
// Summed device time (ms) of the half-transform kernels of the last build (all batches);
// valid once that build has completed.
float oz_last_transform_ms(OzState* o);
// C (+)= A op(B) to FP64 accuracy from the same digit products (A M x K, C M x N, all
// row-major on the device with leading dimensions lda, ldb, ldc; op(B) = B, K x N, or with
// transb op(B) = B^T for B N x K); B is taken in column chunks of op(B) whose digits fit
// GDFJK_OZ_GEMM_CHUNK_GB (default 8).  Returns after the product is complete.
int oz_gemm(OzState* o, const double* A, size_t lda, const double* B, size_t ldb, double* C, size_t ldc, int M, int N,
            int K, int accumulate, cudaStream_t s, std::string& err, int transb = 0);
// error bits raised by the tensor-core kernels since the last call (0 = none); clears them
int oz_error_flag(OzState* o, cudaStream_t s);

}  // namespace gdfjk
