// common.cuh — shared definitions of the GB300 DF-JK engine.
//
// Device layout of B (the metric-contracted 3-index tensor B[Q][m][n], symmetric in mn):
// the nbf x nbf matrix of every Q is cut into 64 x 64 tiles; only tiles (I, J) with I >= J
// that hold at least one Schwarz-significant pair are stored ("stored tiles"), each as a
// dense row-major 64 x 64 block (screened pairs and padding are zero).  Diagonal tiles are
// stored in full (both triangles).  Storage is Q-major:
//     B[((size_t)Q * ntiles + t) * 4096 + r * 64 + c] = B_Q[64*I_t + r][64*J_t + c].
// This keeps every tile a contiguous 32 KB block (bulk copies, coalesced streaming) and
// the whole of one Q contiguous; an upper-triangle tile is read as the transpose of its
// stored mirror.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

namespace gdfjk {

constexpr int TILE = 64;
constexpr int TILE_ELEMS = TILE * TILE;

// device-side error codes written into the handle's flag word (never __trap)
constexpr int DEV_ERR_INDEX = 1;
constexpr int DEV_ERR_WAIT = 2;

// Bounds-checked build (-DGDFJK_BOUNDS_CHECK, `_native.build_jk(bounds_check=True)`): the
// kernels check every bulk-copy source range and global write index against the extent of
// its buffer; a violation raises DEV_ERR_INDEX, prints the first few (code, index, limit)
// triples and skips the access (a producer stops its stream of copies and aborts its block).
// Compiled out otherwise (BCHK is then `true`).
#ifdef GDFJK_BOUNDS_CHECK
static __device__ int g_bounds_reports;  // per translation unit: the first 16 violations are printed
__device__ __forceinline__ bool bounds_check(bool ok, int* err, int code, long long idx, long long lim) {
    if (!ok) {
        atomicOr(err, DEV_ERR_INDEX);
        if (atomicAdd(&g_bounds_reports, 1) < 16)
            printf("GDFJK_BOUNDS code %d block %d thread %d index %lld limit %lld\n", code, (int)blockIdx.x,
                   (int)threadIdx.x, idx, lim);
    }
    return ok;
}
#define BCHK(cond, err, code, idx, lim) ::gdfjk::bounds_check((cond), (err), (code), (long long)(idx), (long long)(lim))
#else
#define BCHK(cond, err, code, idx, lim) true
#endif
// [off, off + len) inside [0, lim) (elements or bytes, as the limit is counted)
#define BRANGE(off, len, lim, err, code) \
    BCHK((size_t)(off) + (size_t)(len) <= (size_t)(lim), err, code, (size_t)(off) + (size_t)(len), lim)

// Codes of the checked sites (printed with the offending index and its limit).
enum BoundsSite {
    BC_TR_LIST = 10,   // emulated half-transform: listed k-block position
    BC_TR_BD = 11,     //   bulk copy of the int8 digits of B
    BC_TR_CD = 12,     //   bulk copy of the BF16 digits of C^T
    BC_TR_X = 13,      //   epilogue: X element
    BC_TR_XMAX = 14,   //   epilogue: group maximum of X
    BC_TR_SA = 15,     //   epilogue: row weight of B
    BC_SX_READ = 20,   // split of X: X read
    BC_SX_WRITE = 21,  //   digit slices written
    BC_SX_SX = 22,     //   group weights
    BC_CT_A = 30,      // emulated contraction: bulk copy of the row operand
    BC_CT_B = 31,      //   bulk copy of the column operand
    BC_CT_S = 32,      //   row / column weights
    BC_CT_OUT = 33,    //   output tile or partial tile
    BC_RED = 40,       // reduction of partial tiles (both forms): tile map and partial reads
    BC_MX_A = 50,      // split-precision GEMM: bulk copy of the A operand
    BC_MX_B = 51,      //   bulk copy of the B operand
    BC_MX_OUT = 52,    //   epilogue write (X blocks or partial tiles)
};

struct TileLayout {
    int nT;          // tiles per dimension
    int ntiles;      // stored tiles
    const int* tI;   // [ntiles]
    const int* tJ;   // [ntiles]
    const int* map;  // [nT*nT]: stored index of (I, J) for I >= J, -1 if absent
};

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

// Record an error message for gdfjk_last_error(NULL) on this thread; returns `code`.
int report_error(int code, const std::string& msg);

// Memory tiers of the large arrays (B and its derived copies): HBM, or pinned Grace memory
// mapped into the GPU's address space, which the kernels read coherently over NVLink-C2C
// (the device pointer is the host pointer).  big_alloc puts `bytes` in host memory when
// `host`, else in HBM; big_free releases either kind.
cudaError_t big_alloc(void** p, size_t bytes, bool host);
void big_free(void* p);
bool is_host_memory(const void* p);

// Every device or pinned allocation of the engine goes through engine_malloc, which
// cudaMalloc's unless a host-side fault injection (gdfjk_debug_refuse_allocations) asks it
// to refuse: it then returns cudaErrorMemoryAllocation without allocating.
cudaError_t engine_malloc(void** p, size_t bytes);
bool alloc_refused();

}  // namespace gdfjk

// kernels (defined in j_kernels.cu / k_fp64.cu); all enqueue on `stream`.
namespace gdfjk {

void launch_relayout_qtri(const double* src, int q0, int nq, int nbf, const TileLayout& L, double* B,
                          cudaStream_t stream);
void launch_pad_C(const double* C, int nbf, int nocc, int ldc, int nbf_pad, int nocc_pad, double* Cpad,
                  cudaStream_t stream);
void launch_density(const double* Cl, const double* Cr, int nbf_pad, int nocc_pad, double* D, cudaStream_t stream);
void launch_weighted_density_tiles(const double* D, int nbf_pad, const TileLayout& L, double* Dw, cudaStream_t stream);
void launch_j_pass1(const double* B, const double* Dw, int naux, const TileLayout& L, double* dq, cudaStream_t stream);
void launch_j_pass2(const double* B, const double* dq, int naux, const TileLayout& L, double* Jt, cudaStream_t stream);
void launch_unpack_tiles(const double* Xt, const TileLayout& L, int nbf, int nbf_pad, double* out, int ld,
                         bool symmetric, cudaStream_t stream);
void launch_k_transform_fp64(const double* B, const double* Cpad, int naux, int nbf_pad, int nocc_pad,
                             const TileLayout& L, double* X, cudaStream_t stream);
void launch_k_contract_fp64(const double* Xl, const double* Xr, int nbf_pad, size_t kdim, bool symmetric,
                            const TileLayout& L, double* Kpart, int nsplit, double* Kt, cudaStream_t stream);
// sum_Q B_Q Y_Q with Y[n][Q][i] (row stride naux*nocc_pad): partial[qblock][m][i]
int back_transform_qblocks(int naux);
void launch_back_transform_fp64(const double* B, const double* Y, int naux, int nbf_pad, int nocc_pad,
                                const TileLayout& L, double* partial, cudaStream_t stream);
int k_contract_splits(int nbf_pad, size_t kdim, bool symmetric);
void launch_unpack_lower_full(const double* Xt, int nT, int nbf, double* out, int ld, cudaStream_t stream);
void launch_copy_out(const double* src, int nbf, int nbf_pad, double* dst, cudaStream_t stream);
// backward.cu
void launch_pad_sym(const double* g, int nbf, int nbf_pad, double* out, cudaStream_t stream);
void launch_gemm_nn_fp64(int M, size_t N, int K, const double* A, size_t lda, const double* Bm, size_t ldb, double alpha,
                         double beta, double* out, size_t ldo, cudaStream_t stream);
// Gamma rows for the naux aux functions of Y (row Q at out + Q*ldo, ldo = 0: nbf(nbf+1)/2),
// packed-triangle columns or col_map's
void launch_gamma(const double* Y, const double* C, const double* gJ, const double* D, const double* dq,
                  const double* gq, int naux, int nbf, int nbf_pad, int nocc_pad, const TileLayout& L, double* out,
                  cudaStream_t stream, size_t ldo = 0, const long long* col_map = nullptr);
// the batched backward's tensor-core Gamma: Y to Q-major rows, then the listed pairs of P
void launch_y_to_qmajor(const double* Y, int nq, int qs0, int nqs, int nbf_pad, int nocc_pad, double* Yq,
                        cudaStream_t stream);
void launch_gamma_gather(const double* P, int nqs, int nbf_pad, const int* pm, const int* pn, const int* pcol,
                         size_t npairs, const double* gJ, const double* D, const double* dq, const double* gq,
                         double* out, size_t ldo, cudaStream_t stream);
void launch_reduce_blocks(const double* part, int nblk, size_t n, double alpha, double beta, double* out,
                          cudaStream_t stream);
void launch_copy_rect(const double* src, int nbf, int nocc, int nocc_pad, double* dst, int ldd, cudaStream_t stream);
void launch_finite_check(const double* a, size_t n, int* flag, cudaStream_t stream);

}  // namespace gdfjk
