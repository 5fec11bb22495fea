// backward.cu — reverse mode of one lr-symmetric DF-JK build (the differentiation form).
//
// Forward: D = C C^T, d_Q = sum_mn B_Q,mn D_mn, J = sum_Q B_Q d_Q, X_Q = B_Q C,
//          K = sum_Q X_Q X_Q^T.
// Given upstream gJ = dE/dJ, gK = dE/dK (symmetrised), with g_Q = sum_mn B_Q,mn gJ_mn and
// Y_Q = gK X_Q:
//   dE/dB_Q  = gJ d_Q + g_Q D + Y_Q C^T + C Y_Q^T                     (Gamma, B-space)
//   dE/dC    = 2 J[gJ] C + 2 sum_Q B_Q Y_Q,    J[gJ] = sum_Q B_Q g_Q
// These are the B-space counterparts of the densities psi4's DFJKGrad builds before it
// contracts with derivative integrals (psi4/src/psi4/scfgrad/jk_grad.cc:294-832: c_A, d_A,
// (A|ij), V_AB, (A|mn)_K); X_Q is recomputed here, never stored between calls.
#include <algorithm>

#include "common.cuh"

namespace gdfjk {

// out[m][n] = (g[m][n] + g[n][m]) / 2 for m, n < nbf, 0 in the padding.
__global__ void pad_sym_kernel(const double* __restrict__ g, int nbf, int nbf_pad, double* __restrict__ out) {
    size_t n = (size_t)nbf_pad * nbf_pad;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        int m = (int)(e / nbf_pad), k = (int)(e % nbf_pad);
        out[e] = (m < nbf && k < nbf) ? 0.5 * (g[(size_t)m * nbf + k] + g[(size_t)k * nbf + m]) : 0.0;
    }
}

void launch_pad_sym(const double* g, int nbf, int nbf_pad, double* out, cudaStream_t stream) {
    size_t n = (size_t)nbf_pad * nbf_pad;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    pad_sym_kernel<<<blocks, 256, 0, stream>>>(g, nbf, nbf_pad, out);
}

// out[m][j] = alpha * sum_k A[m][k] Bm[k][j] + beta * out[m][j]
// M % 64 == 0, N % 32 == 0, K % 32 == 0.  grid (N/32, M/64), 128 threads.
__global__ void __launch_bounds__(128) gemm_nn_fp64_kernel(int K, const double* __restrict__ A, size_t lda,
                                                           const double* __restrict__ Bm, size_t ldb, double alpha,
                                                           double beta, double* __restrict__ out, size_t ldo) {
    __shared__ double As[32][TILE + 1];
    __shared__ double Bs[32][32];
    int m0 = blockIdx.y * TILE;
    size_t j0 = (size_t)blockIdx.x * 32;
    int tid = threadIdx.x, ty = tid / 8, tx = tid % 8;
    double acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += 32) {
        for (int e = tid; e < 32 * TILE; e += 128) {
            int r = e / 32, kk = e % 32;
            As[kk][r] = __ldg(A + (size_t)(m0 + r) * lda + k0 + kk);
        }
        for (int e = tid; e < 32 * 32; e += 128) {
            int kk = e / 32, j = e % 32;
            Bs[kk][j] = __ldg(Bm + (size_t)(k0 + kk) * ldb + j0 + j);
        }
        __syncthreads();
#pragma unroll 8
        for (int kk = 0; kk < 32; ++kk) {
            double a[4], b[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                a[u] = As[kk][ty * 4 + u];
                b[u] = Bs[kk][tx * 4 + u];
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            double* o = out + (size_t)(m0 + ty * 4 + u) * ldo + j0 + tx * 4 + v;
            *o = alpha * acc[u][v] + (beta != 0.0 ? beta * *o : 0.0);
        }
}

void launch_gemm_nn_fp64(int M, size_t N, int K, const double* A, size_t lda, const double* Bm, size_t ldb, double alpha,
                         double beta, double* out, size_t ldo, cudaStream_t stream) {
    if (M == 0 || N == 0) return;
    // grid.x can reach naux*nocc/32 (< 2^31): fine for x
    dim3 grid((unsigned)(N / 32), M / TILE);
    gemm_nn_fp64_kernel<<<grid, 128, 0, stream>>>(K, A, lda, Bm, ldb, alpha, beta, out, ldo);
}

// Gamma for the stored tile t and auxiliary index Q (blockIdx = (t, Q)), written to
// out[Q*ldo + col] with col = m(m+1)/2 + n for m >= n, or col_map[m(m+1)/2 + n] (entries < 0
// are not stored), x2 off the diagonal.  Y[m][Q][i], C[m][i]; dq, gq indexed by the same Q.
__global__ void __launch_bounds__(256) gamma_kernel(const double* __restrict__ Y, const double* __restrict__ C,
                                                    const double* __restrict__ gJ, const double* __restrict__ D,
                                                    const double* __restrict__ dq, const double* __restrict__ gq,
                                                    int naux, int nbf, int nbf_pad, int nocc_pad,
                                                    const int* __restrict__ tI, const int* __restrict__ tJ,
                                                    double* __restrict__ out, size_t ldo,
                                                    const long long* __restrict__ col_map) {
    __shared__ double Ym[16][TILE + 1], Cm[16][TILE + 1], Yn[16][TILE + 1], Cn[16][TILE + 1];
    int t = blockIdx.x, Q = blockIdx.y;
    int I = tI[t], J = tJ[t];
    int tid = threadIdx.x, ty = tid / 16, tx = tid % 16;
    double acc[4][4] = {};
    for (int i0 = 0; i0 < nocc_pad; i0 += 16) {
        for (int e = tid; e < 16 * TILE; e += 256) {
            int r = e / 16, kk = e % 16;
            size_t mi = (size_t)I * TILE + r, ni = (size_t)J * TILE + r;
            Ym[kk][r] = __ldg(Y + (mi * naux + Q) * nocc_pad + i0 + kk);
            Cm[kk][r] = __ldg(C + mi * nocc_pad + i0 + kk);
            Yn[kk][r] = __ldg(Y + (ni * naux + Q) * nocc_pad + i0 + kk);
            Cn[kk][r] = __ldg(C + ni * nocc_pad + i0 + kk);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < 16; ++kk) {
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                double ym = Ym[kk][ty * 4 + u], cm = Cm[kk][ty * 4 + u];
#pragma unroll
                for (int v = 0; v < 4; ++v)
                    acc[u][v] = fma(ym, Cn[kk][tx * 4 + v], fma(cm, Yn[kk][tx * 4 + v], acc[u][v]));
            }
        }
        __syncthreads();
    }
    double d = dq[Q], g = gq[Q];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            int m = I * TILE + ty * 4 + u, n = J * TILE + tx * 4 + v;
            if (m >= nbf || n >= nbf || m < n) continue;
            size_t mn = (size_t)m * nbf_pad + n;
            double val = acc[u][v] + gJ[mn] * d + g * D[mn];
            long long col = (long long)m * (m + 1) / 2 + n;
            if (col_map) {
                col = col_map[col];
                if (col < 0) continue;
            }
            out[(size_t)Q * ldo + (size_t)col] = (m > n ? 2.0 : 1.0) * val;
        }
}

void launch_gamma(const double* Y, const double* C, const double* gJ, const double* D, const double* dq,
                  const double* gq, int naux, int nbf, int nbf_pad, int nocc_pad, const TileLayout& L, double* out,
                  cudaStream_t stream, size_t ldo, const long long* col_map) {
    if (L.ntiles == 0 || naux == 0) return;
    if (ldo == 0) ldo = (size_t)nbf * (nbf + 1) / 2;
    dim3 grid(L.ntiles, naux);
    gamma_kernel<<<grid, 256, 0, stream>>>(Y, C, gJ, D, dq, gq, naux, nbf, nbf_pad, nocc_pad, L.tI, L.tJ, out, ldo,
                                           col_map);
}

// Y (layout [m][Q][i], nq aux functions) -> Yq[Q'][m][i] for Q = qs0 + Q', Q' < nqs
__global__ void y_to_qmajor_kernel(const double* __restrict__ Y, int nq, int qs0, int nqs, int nbf_pad, int nocc_pad,
                                   double* __restrict__ Yq) {
    const size_t n = (size_t)nqs * nbf_pad * nocc_pad;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e % nocc_pad);
        const size_t r = e / nocc_pad;
        const int m = (int)(r % nbf_pad), q = (int)(r / nbf_pad);
        Yq[e] = Y[((size_t)m * nq + qs0 + q) * nocc_pad + i];
    }
}

void launch_y_to_qmajor(const double* Y, int nq, int qs0, int nqs, int nbf_pad, int nocc_pad, double* Yq,
                        cudaStream_t stream) {
    const size_t n = (size_t)nqs * nbf_pad * nocc_pad;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    y_to_qmajor_kernel<<<std::max(blocks, 1), 256, 0, stream>>>(Y, nq, qs0, nqs, nbf_pad, nocc_pad, Yq);
}

// Gamma from P[Q][m][n] = sum_i Y_Q[m][i] C[n][i] (a dense product): for each listed pair
// (m >= n, column col) out[Q*ldo + col] = (2 if m > n) (P[m][n] + P[n][m] + gJ_mn d_Q + g_Q D_mn),
// the same value gamma_kernel forms from Y and C directly.
__global__ void gamma_gather_kernel(const double* __restrict__ P, int nqs, int nbf_pad, const int* __restrict__ pm,
                                    const int* __restrict__ pn, const int* __restrict__ pcol, size_t npairs,
                                    const double* __restrict__ gJ, const double* __restrict__ D,
                                    const double* __restrict__ dq, const double* __restrict__ gq,
                                    double* __restrict__ out, size_t ldo) {
    const size_t n = npairs * nqs;
    const size_t np2 = (size_t)nbf_pad * nbf_pad;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        const int q = (int)(e / npairs);
        const size_t k = e % npairs;
        const size_t m = (size_t)pm[k], nn = (size_t)pn[k];
        const double* PQ = P + (size_t)q * np2;
        const size_t mn = m * nbf_pad + nn;
        const double v = PQ[mn] + PQ[nn * nbf_pad + m] + gJ[mn] * dq[q] + gq[q] * D[mn];
        out[(size_t)q * ldo + (size_t)pcol[k]] = (m > nn ? 2.0 : 1.0) * v;
    }
}

void launch_gamma_gather(const double* P, int nqs, int nbf_pad, const int* pm, const int* pn, const int* pcol,
                         size_t npairs, const double* gJ, const double* D, const double* dq, const double* gq,
                         double* out, size_t ldo, cudaStream_t stream) {
    const size_t n = npairs * nqs;
    if (n == 0) return;
    const int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 32);
    gamma_gather_kernel<<<blocks, 256, 0, stream>>>(P, nqs, nbf_pad, pm, pn, pcol, npairs, gJ, D, dq, gq, out, ldo);
}

// out[e] = alpha * sum_{b < nblk} part[b*n + e] + beta * out[e]   (fixed order)
__global__ void reduce_blocks_kernel(const double* __restrict__ part, int nblk, size_t n, double alpha, double beta,
                                     double* __restrict__ out) {
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        double s = 0.0;
        for (int b = 0; b < nblk; ++b) s += part[(size_t)b * n + e];
        out[e] = alpha * s + (beta != 0.0 ? beta * out[e] : 0.0);
    }
}

void launch_reduce_blocks(const double* part, int nblk, size_t n, double alpha, double beta, double* out,
                          cudaStream_t stream) {
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    if (blocks < 1) blocks = 1;
    reduce_blocks_kernel<<<blocks, 256, 0, stream>>>(part, nblk, n, alpha, beta, out);
}

// dst[m*ldd + i] = src[m*nocc_pad + i] for m < nbf, i < nocc
__global__ void copy_rect_kernel(const double* __restrict__ src, int nbf, int nocc, int nocc_pad, double* __restrict__ dst,
                                 int ldd) {
    size_t n = (size_t)nbf * nocc;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        int m = (int)(e / nocc), i = (int)(e % nocc);
        dst[(size_t)m * ldd + i] = src[(size_t)m * nocc_pad + i];
    }
}

void launch_copy_rect(const double* src, int nbf, int nocc, int nocc_pad, double* dst, int ldd, cudaStream_t stream) {
    size_t n = (size_t)nbf * nocc;
    if (n == 0) return;
    int blocks = (int)std::min<size_t>((n + 255) / 256, 152 * 16);
    copy_rect_kernel<<<blocks, 256, 0, stream>>>(src, nbf, nocc, nocc_pad, dst, ldd);
}

}  // namespace gdfjk
