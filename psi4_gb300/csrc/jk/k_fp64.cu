// k_fp64.cu — FP64 exchange (K) kernels of the GB300 DF-JK engine.
//
// Restates DFHelper::compute_K (psi4/src/psi4/lib3index/dfhelper.cc:3350-3377):
//   half-transform  X[m][Q][i] = sum_n B_Q,mn C_ni          (first_transform_pQq, :2162-2186)
//   contraction     K_mn       = sum_{Q,i} X[m][Q,i] X[n][Q,i]   (C_DGEMM('N','T'), :3374)
// GB300's FP64 rate is about 1.1 TFLOP/s (measured cuBLAS DGEMM), i.e. a few FP64 FMAs per
// clock per SM, so both FP64 kernels are FMA-bound by a wide margin: a 64-row x 32-column
// register-tiled block with shared-memory staging keeps the FP64 pipe busy while reading
// B once per output column block.  The contraction is symmetric (lower tiles only when
// C_left == C_right) and split along its long inner dimension (naux * nocc) with a
// fixed-order reduction of the partial tiles, so results are reproducible.
#include "common.cuh"

namespace gdfjk {

// ---------------------------------------------------------------- half-transform
// grid (nT * nib, nQblocks), 128 threads; a block computes 64 rows (tile I) x 32 columns.
// Per-Q mode (ACCUM = false): out[(m*naux + Q)*nocc_pad + i] = sum_n B_Q,mn R_Q[n][i] for the
// block's single Q = blockIdx.y.  Accumulating mode (ACCUM = true): the block sums over
// Q in [blockIdx.y*qper, ...) and writes out[(blockIdx.y*nbf_pad + m)*nocc_pad + i].
// The right operand of Q is R_Q[n][i] = R[n*ldr + Q*qoff + i] (qoff = 0: one C for all Q).
constexpr int KT_BN = 32;
template <bool ACCUM>
__global__ void __launch_bounds__(128) k_transform_fp64_kernel(const double* __restrict__ B,
                                                               const double* __restrict__ R, size_t ldr, size_t qoff,
                                                               int naux, int nocc_pad, int nbf_pad, int qper, int nT,
                                                               int ntiles, const int* __restrict__ map,
                                                               double* __restrict__ out) {
    constexpr int KH = 32;                 // k depth staged per step (half a tile)
    __shared__ double As[KH][TILE + 1];   // As[k][r]
    __shared__ double Cs[KH][KT_BN];
    int nib = nocc_pad / KT_BN;
    int I = blockIdx.x / nib, ib = blockIdx.x % nib;
    int q_begin = ACCUM ? blockIdx.y * qper : blockIdx.y;
    int q_end = ACCUM ? min(naux, q_begin + qper) : q_begin + 1;
    int tid = threadIdx.x;
    int ty = tid / 8, tx = tid % 8;  // 16 x 8 threads, 4 x 4 outputs each
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) acc[a][b] = 0.0;
    for (int Q = q_begin; Q < q_end; ++Q) {
        const double* RQ = R + (size_t)Q * qoff;
        for (int J = 0; J < nT; ++J) {
            int t;
            bool trans;
            if (I >= J) {
                t = map[I * nT + J];
                trans = false;
            } else {
                t = map[J * nT + I];
                trans = true;
            }
            if (t < 0) continue;  // block-uniform
            const double* T = B + ((size_t)Q * ntiles + t) * TILE_ELEMS;
            for (int kh = 0; kh < TILE; kh += KH) {
                if (!trans) {
                    // A[r][k] = T[r][k]
                    for (int e = tid; e < KH * TILE; e += 128) {
                        int r = e / KH, kk = e % KH;
                        As[kk][r] = __ldg(T + r * TILE + kh + kk);
                    }
                } else {
                    // A[r][k] = T[k][r]
                    for (int e = tid; e < KH * TILE; e += 128) {
                        int kk = e / TILE, r = e % TILE;
                        As[kk][r] = __ldg(T + (kh + kk) * TILE + r);
                    }
                }
                for (int e = tid; e < KH * KT_BN; e += 128) {
                    int k = e / KT_BN, j = e % KT_BN;
                    Cs[k][j] = __ldg(RQ + (size_t)(J * TILE + kh + k) * ldr + ib * KT_BN + j);
                }
                __syncthreads();
#pragma unroll 8
                for (int k = 0; k < KH; ++k) {
                    double a[4], c[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) {
                        a[u] = As[k][ty * 4 + u];
                        c[u] = Cs[k][tx * 4 + u];
                    }
#pragma unroll
                    for (int u = 0; u < 4; ++u)
#pragma unroll
                        for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], c[v], acc[u][v]);
                }
                __syncthreads();
            }
        }
    }
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        size_t m = (size_t)I * TILE + ty * 4 + u;
        double* dst = ACCUM ? out + ((size_t)blockIdx.y * nbf_pad + m) * nocc_pad + ib * KT_BN + tx * 4
                            : out + (m * naux + q_begin) * nocc_pad + ib * KT_BN + tx * 4;
#pragma unroll
        for (int v = 0; v < 4; ++v) dst[v] = acc[u][v];
    }
}

void launch_k_transform_fp64(const double* B, const double* Cpad, int naux, int nbf_pad, int nocc_pad,
                             const TileLayout& L, double* X, cudaStream_t stream) {
    if (nocc_pad == 0 || naux == 0) return;
    dim3 grid(L.nT * (nocc_pad / KT_BN), naux);
    k_transform_fp64_kernel<false><<<grid, 128, 0, stream>>>(B, Cpad, nocc_pad, 0, naux, nocc_pad, nbf_pad, 1, L.nT,
                                                             L.ntiles, L.map, X);
}

int back_transform_qblocks(int naux) { return naux < 64 ? naux : 64; }

void launch_back_transform_fp64(const double* B, const double* Y, int naux, int nbf_pad, int nocc_pad,
                                const TileLayout& L, double* partial, cudaStream_t stream) {
    if (nocc_pad == 0 || naux == 0) return;
    int nqb = back_transform_qblocks(naux);
    int qper = (naux + nqb - 1) / nqb;
    nqb = (naux + qper - 1) / qper;
    dim3 grid(L.nT * (nocc_pad / KT_BN), nqb);
    k_transform_fp64_kernel<true><<<grid, 128, 0, stream>>>(B, Y, (size_t)naux * nocc_pad, nocc_pad, naux, nocc_pad,
                                                            nbf_pad, qper, L.nT, L.ntiles, L.map, partial);
}

// ---------------------------------------------------------------- contraction
// grid (nout, nsplit), 256 threads; block computes a 64x64 partial K tile over one k range.
constexpr int KC_BK = 16;
__global__ void __launch_bounds__(256) k_contract_fp64_kernel(const double* __restrict__ Xl,
                                                              const double* __restrict__ Xr, size_t kdim, int nT,
                                                              int symmetric, size_t kchunk, int nout,
                                                              double* __restrict__ Kpart) {
    __shared__ double As[KC_BK][TILE + 1];
    __shared__ double Bs[KC_BK][TILE + 1];
    int b = blockIdx.x, s = blockIdx.y;
    int I, J;
    if (symmetric) {
        // b = I(I+1)/2 + J, J <= I
        I = (int)((sqrt(8.0 * b + 1.0) - 1.0) * 0.5);
        while (I * (I + 1) / 2 > b) --I;
        while ((I + 1) * (I + 2) / 2 <= b) ++I;
        J = b - I * (I + 1) / 2;
    } else {
        I = b / nT;
        J = b % nT;
    }
    size_t k_begin = (size_t)s * kchunk;
    size_t k_end = k_begin + kchunk;
    if (k_end > kdim) k_end = kdim;
    int tid = threadIdx.x;
    int ty = tid / 16, tx = tid % 16;
    const double* A0 = Xl + (size_t)I * TILE * kdim;
    const double* B0 = Xr + (size_t)J * TILE * kdim;
    double acc[4][4];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][c] = 0.0;
    for (size_t k0 = k_begin; k0 < k_end; k0 += KC_BK) {
        for (int e = tid; e < TILE * KC_BK; e += 256) {
            int r = e / KC_BK, kk = e % KC_BK;
            size_t k = k0 + kk;
            bool in = k < k_end;
            As[kk][r] = in ? __ldg(A0 + (size_t)r * kdim + k) : 0.0;
            Bs[kk][r] = in ? __ldg(B0 + (size_t)r * kdim + k) : 0.0;
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < KC_BK; ++kk) {
            double a[4], c[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = As[kk][ty * 4 + u];
                c[u] = Bs[kk][tx * 4 + u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], c[v], acc[u][v]);
        }
        __syncthreads();
    }
    double* dst = Kpart + ((size_t)s * nout + b) * TILE_ELEMS;
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) dst[(ty * 4 + u) * TILE + tx * 4 + v] = acc[u][v];
}

__global__ void k_reduce_kernel(const double* __restrict__ Kpart, int nsplit, size_t n, double* __restrict__ Kt) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int k = 0; k < nsplit; ++k) s += Kpart[(size_t)k * n + e];
        Kt[e] = s;
    }
}

int k_contract_splits(int nbf_pad, size_t kdim, bool symmetric) {
    int nT = nbf_pad / TILE;
    int nout = symmetric ? nT * (nT + 1) / 2 : nT * nT;
    // aim for ~8 blocks per SM in flight, at least 1024 k per split
    long want = (152L * 8 + nout - 1) / nout;
    long maxs = (long)((kdim + 1023) / 1024);
    if (want > maxs) want = maxs;
    if (want < 1) want = 1;
    if (want > 256) want = 256;
    return (int)want;
}

void launch_k_contract_fp64(const double* Xl, const double* Xr, int nbf_pad, size_t kdim, bool symmetric,
                            const TileLayout& L, double* Kpart, int nsplit, double* Kt, cudaStream_t stream) {
    (void)L;
    int nT = nbf_pad / TILE;
    int nout = symmetric ? nT * (nT + 1) / 2 : nT * nT;
    size_t kchunk = (kdim + nsplit - 1) / nsplit;
    kchunk = (kchunk + KC_BK - 1) / KC_BK * KC_BK;
    dim3 grid(nout, nsplit);
    k_contract_fp64_kernel<<<grid, 256, 0, stream>>>(Xl, Xr, kdim, nT, symmetric ? 1 : 0, kchunk, nout, Kpart);
    size_t n = (size_t)nout * TILE_ELEMS;
    int blocks = (int)((n + 255) / 256);
    if (blocks > 152 * 16) blocks = 152 * 16;
    k_reduce_kernel<<<blocks, 256, 0, stream>>>(Kpart, nsplit, n, Kt);
}

}  // namespace gdfjk
