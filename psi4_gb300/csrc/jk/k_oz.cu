// k_oz.cu — FP64-accurate exchange on the BF16 tensor cores (digit-split, "Ozaki" scheme).
//
// K = sum_Q B_Q C C^T B_Q to FP64 accuracy, with every multiply-add on tcgen05 BF16 MMAs
// (Ozaki, Ogita, Oishi & Rump 2012, "Error-free transformations of matrix multiplication by
// using fast routines of matrix multiplication and its applications"; here with balanced
// 7-bit digits so that BF16 holds each digit exactly).
//
// Digits.  A row (or row chunk) with |x| < 2^E is written in fixed point as
//     v = round(x * 2^(47-E)),  |v| <= 2^47,   v = sum_{s=0..6} d_s 2^(7(6-s)),  d_s in [-64, 63]
// so x = 2^(E-5) * sum_s g_s (+ |error| <= 2^(E-48)) with the slice values g_s = d_s 2^(-7s),
// each exact in BF16.  The digits come from integer arithmetic on the IEEE bit pattern (no
// FP64 instruction: this GPU's FP64 pipe runs at ~1/60 of its FP32 rate).
//
// Products.  (x y) = 2^(Ex+Ey-10) sum_{s+t<=6} g_s h_t  (28 slice pairs; the level-7 pairs
// dropped and the digit remainders are ~2^-44 of |x|max|y|max per term).  Pairs are grouped
// by level L = s+t into six tensor-memory accumulators: L = 0..4 each on its own, as sums of
// integers times one power of two, exact in FP32 while a partial sum stays below 2^24 units
// (provably for L <= 3 in a run of at most 1024 terms: 4 pairs x 1024 x 64^2 = 2^24; level 4
// in all but adversarial digit patterns), and the tail L = 5, 6 prescaled.  The tensor cores'
// FP32 accumulation rounds toward zero: on an inexact accumulator that holds positive terms
// (the squares on the diagonal of K) the truncations add up to a bias, ~2^-36 relative with a
// level-4 tail; with the tail at levels 5-6 it is 2^7 smaller.  The epilogue adds the six in
// double-float (FP32 pairs).
//
//   half-transform   X[m][(Q,i)] = sum_n B_Q[m][n] C[n][i]      A = digits of B (int8 in HBM,
//                    converted to BF16 slice values by four converter warps that write them
//                    straight into tensor memory), B = digits of C^T (BF16, shared memory);
//                    one item = (Q, 128 rows, a chunk of <= 80 columns), k in runs of <= 2048;
//                    X out in double-float plus a row max per group of Q.
//   split            X -> BF16 digit slices with one exponent per (row, group of Q), a group
//                    being <= 1024 contraction terms.
//   contraction      K[m][n] = sum_groups 2^(E_m+E_n-10) sum_pairs ... : 128 x 64 tiles of the
//                    lower triangle; both operands from shared memory; the pairs of the exact
//                    levels of one A slice issued as one wide MMA over the level regions, which
//                    lie side by side in TMEM (19 MMAs per 16 k instead of 28);
//                    one accumulation run per group, drained into a double-float running sum
//                    in registers; split over groups; FP64 partials summed in a fixed order.
// In both GEMMs one pipeline stage holds every digit slice of one 32-deep k block, and the
// MMA issuers walk the A slices j = 0..6 (in the half-transform each from its TMEM slot)
// against B slices t = 0..6-j, accumulator min(j + t, last); the half-transform has two
// issuing threads, one for the exact levels' accumulators and one for the tail's.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>
#include <vector>

#include "block_lists.h"
#include "gdfjk.h"
#include "oz.cuh"
#include "tc_common.cuh"

namespace gdfjk {
namespace oz {

constexpr int MM = 128;                      // tile rows (MMA M)
constexpr int MK = 32;                       // k per pipeline stage (one 64-byte row of BF16)
constexpr int NSL = 7;                       // digit slices
constexpr int NACC = 6;                      // accumulators: levels 0..4 and the tail (5, 6)
constexpr int I8_SLICE = MM * MK;            // bytes of one int8 digit slice of a 128 x 32 block
constexpr int BF_SLICE = MM * MK * 2;        // bytes of one BF16 slice of a 128 x 32 block
constexpr int I8_BLOCK = NSL * I8_SLICE;     // 28 KB: all slices of one 128 x 32 block of B
constexpr int E_EMPTY = -100000;             // exponent of an all-zero row
constexpr int SMEM_BUDGET = 224 * 1024;
constexpr int SMEM_RESERVE = 2048;
constexpr int TR_THREADS = 480;              // producer, 2 MMA, 8 epilogue warps, 4 converter warps
constexpr int CT_N = 64;                     // contraction tile columns
constexpr int TR_MAX_N = 80;                 // half-transform accumulator columns
constexpr int RUN_K = 1024;                  // contraction terms per accumulation run (levels 0-3 exact)
constexpr int TR_RUN_K = 2048;               // half-transform terms per run (levels 0-1 exact for any digits)
static_assert(tc::SWZ == 64, "digit slices are laid out for the 64-byte swizzle");

// offset added to v so that every base-128 digit field of u = v + OFF is d_s + 64 in [0, 127]
constexpr unsigned long long DIGIT_OFF =
    64ull * (1ull + (1ull << 7) + (1ull << 14) + (1ull << 21) + (1ull << 28) + (1ull << 35) + (1ull << 42));

// E with |x| < 2^E for the largest magnitude |x| whose bits are given (sign cleared)
__device__ __forceinline__ int exp_of_max_d(unsigned long long bits) {
    if (bits == 0) return E_EMPTY;
    int ex = (int)(bits >> 52);
    if (ex == 0) ex = 1;
    return ex - 1022;
}
__device__ __forceinline__ int exp_of_max_f(unsigned bits) {
    if (bits == 0) return E_EMPTY;
    int ex = (int)(bits >> 23);
    if (ex == 0) ex = 1;
    return ex - 126;
}
// Non-finite inputs (Inf / NaN bits in a maximum) would turn into finite digit garbage, so
// the exponent kernels raise the numeric error bit instead (the host returns GDFJK_ERR_NUMERIC).
constexpr unsigned long long NONFINITE_BITS = 0x7FF0000000000000ull;
constexpr int DEV_ERR_NUMERIC = 4;

// 2^(E-5) as a float (the slice weight of a row); 0 for empty rows or below the normal range
__device__ __forceinline__ float scale_of(int E) {
    if (E == E_EMPTY) return 0.f;
    int b = E - 5 + 127;
    if (b <= 0) return 0.f;
    if (b > 254) b = 254;
    return __int_as_float(b << 23);
}

// round(x * 2^(47-E)) for |x| < 2^E, from the bit pattern
__device__ __forceinline__ long long fix_d(double x, int E) {
    if (E == E_EMPTY) return 0;
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    int ex = (int)((b >> 52) & 0x7FF);
    unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
    if (ex)
        mant |= 1ull << 52;
    else
        ex = 1;
    int r = 1028 + E - ex;  // >= 6 because |x| < 2^E
    unsigned long long v = r >= 64 ? 0ull : ((mant + (1ull << (r - 1))) >> r);
    return (b >> 63) ? -(long long)v : (long long)v;
}
__device__ __forceinline__ long long fix_f(float x, int E) {
    if (E == E_EMPTY) return 0;
    unsigned b = __float_as_uint(x);
    int ex = (int)((b >> 23) & 255);
    unsigned long long mant = b & 0x7FFFFFu;
    if (ex)
        mant |= 0x800000u;
    else
        ex = 1;
    int sh = ex - 103 - E;  // <= 23 because |x| < 2^E
    unsigned long long v;
    if (sh >= 0) {
        v = mant << sh;
    } else {
        int r = -sh;
        v = r >= 40 ? 0ull : ((mant + (1ull << (r - 1))) >> r);
    }
    return (b >> 31) ? -(long long)v : (long long)v;
}
// digit field of slice s (0 = most significant) of u = v + DIGIT_OFF
__device__ __forceinline__ uint32_t digit_field(unsigned long long u, int s) {
    return (uint32_t)(u >> (7 * (NSL - 1 - s))) & 127u;
}

// The same with NS digits (the general product uses eight): v = round(x 2^(7 NS - 2 - E)),
// |v| <= 2^(7 NS - 2), so that x = 2^(E-5) sum_s d_s 2^(-7s) whatever NS is.
template <int NS>
__device__ __forceinline__ long long fix_dn(double x, int E) {
    if (E == E_EMPTY) return 0;
    unsigned long long b = (unsigned long long)__double_as_longlong(x);
    int ex = (int)((b >> 52) & 0x7FF);
    unsigned long long mant = b & 0xFFFFFFFFFFFFFull;
    if (ex)
        mant |= 1ull << 52;
    else
        ex = 1;
    const int r = 1075 - (7 * NS - 2) + E - ex;  // >= 6 - 7 (NS - 7) because |x| < 2^E
    unsigned long long v;
    if (r <= 0)
        v = mant << (-r);
    else
        v = r >= 64 ? 0ull : ((mant + (1ull << (r - 1))) >> r);
    return (b >> 63) ? -(long long)v : (long long)v;
}
template <int NS>
__device__ __forceinline__ unsigned long long digit_off() {
    unsigned long long o = 0;
#pragma unroll
    for (int s = 0; s < NS; ++s) o = (o << 7) | 64ull;
    return o;
}
template <int NS>
__device__ __forceinline__ uint32_t digit_field_n(unsigned long long u, int s) {
    return (uint32_t)(u >> (7 * (NS - 1 - s))) & 127u;
}
// BF16 bits of the slice value (f - 64) * 2^(-7s), exact; w = 2^(-7s)
__device__ __forceinline__ uint32_t field_bf16(uint32_t f, float w) {
    float g = fmaf(__uint_as_float(0x4B000000u | f), w, -8388672.0f * w);
    return __float_as_uint(g) >> 16;
}
__device__ __forceinline__ float slice_weight(int s) { return __int_as_float((127 - 7 * s) << 23); }

// ---------------------------------------------------------------- digits of B (once per upload)
// Row maxima of |B_Q[m][.]| over both triangles from the stored tiles: rows of a stored tile
// (I, J) belong to rows 64I+r, and for I != J its columns to rows 64J+c.
__global__ void oz_rowmax_kernel(const double* __restrict__ B, int ntiles, const int* __restrict__ tI,
                                 const int* __restrict__ tJ, int nbf_p, unsigned long long* __restrict__ rowmax,
                                 int* __restrict__ err) {
    const size_t qt = blockIdx.x;  // Q * ntiles + t
    const int Q = (int)(qt / ntiles), t = (int)(qt % ntiles);
    const int I = tI[t], J = tJ[t];
    const double* tile = B + qt * TILE_ELEMS;
    __shared__ unsigned long long colpart[4][TILE];
    {
        // rows: 4 threads per row, 16 columns each
        int r = threadIdx.x / 4, part = threadIdx.x % 4;
        unsigned long long mx = 0;
        for (int c = part * 16; c < part * 16 + 16; ++c) {
            unsigned long long b = (unsigned long long)__double_as_longlong(tile[r * TILE + c]) & 0x7FFFFFFFFFFFFFFFull;
            mx = b > mx ? b : mx;
        }
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 1));
        mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, 2));
        if (part == 0 && mx) atomicMax(&rowmax[(size_t)Q * nbf_p + I * TILE + r], mx);
        if (part == 0 && mx >= NONFINITE_BITS) atomicOr(err, DEV_ERR_NUMERIC);
    }
    if (I != J) {
        int c = threadIdx.x % TILE, part = threadIdx.x / TILE;
        unsigned long long mx = 0;
        for (int r = part * 16; r < part * 16 + 16; ++r) {
            unsigned long long b = (unsigned long long)__double_as_longlong(tile[r * TILE + c]) & 0x7FFFFFFFFFFFFFFFull;
            mx = b > mx ? b : mx;
        }
        colpart[part][c] = mx;
        __syncthreads();
        if (threadIdx.x < TILE) {
            unsigned long long m2 = max(max(colpart[0][c], colpart[1][c]), max(colpart[2][c], colpart[3][c]));
            if (m2) atomicMax(&rowmax[(size_t)Q * nbf_p + J * TILE + c], m2);
            if (m2 >= NONFINITE_BITS) atomicOr(err, DEV_ERR_NUMERIC);
        }
    }
}

// Int8 digit fields of B, one 28 KB block per (Q, listed (128-row block, 32-wide k block)):
// [slice 7][row 128][k 32] of (d_s + 64).  blockIdx.x = Q * nnz + b; 256 threads.  Only the
// blocks that touch a stored tile are listed (blk_mb/blk_kb, grouped by row block).
// The 128 x 32 FP64 window is staged in shared memory from the stored tiles (lower tiles
// row-wise, upper ones through their stored mirror column-wise, both coalesced).
__global__ void __launch_bounds__(256) oz_split_B_kernel(const double* __restrict__ B, int nbf, int nT, int ntiles,
                                                         const int* __restrict__ map, int nbf_p, int nnz,
                                                         const int* __restrict__ blk_mb, const int* __restrict__ blk_kb,
                                                         const int* __restrict__ mb_ptr,
                                                         const unsigned long long* __restrict__ rowmax,
                                                         float* __restrict__ sA, uint8_t* __restrict__ Bd) {
    const size_t id = blockIdx.x;
    const int b = (int)(id % nnz);
    const int Q = (int)(id / nnz);
    const int mb = blk_mb[b], kb = blk_kb[b];
    __shared__ double win[MM][MK + 1];
    __shared__ int Es[MM];
    const int J = (kb * MK) / TILE, c0 = (kb * MK) % TILE;
    for (int h = 0; h < 2; ++h) {
        const int I = mb * 2 + h;
        int t = -1;
        if (I < nT && J < nT) t = I >= J ? map[I * nT + J] : map[J * nT + I];
        for (int e = threadIdx.x; e < TILE * MK; e += blockDim.x) {
            double v = 0.0;
            int r, c;
            if (I >= J) {  // stored as rows r (of 64), columns c0 + c
                r = e / MK;
                c = e % MK;
                if (t >= 0) v = B[((size_t)Q * ntiles + t) * TILE_ELEMS + r * TILE + c0 + c];
            } else {  // stored mirror (J, I): element (m, n) at [n % 64][m % 64]
                c = e / TILE;
                r = e % TILE;
                if (t >= 0) v = B[((size_t)Q * ntiles + t) * TILE_ELEMS + (c0 + c) * TILE + r];
            }
            const int m = I * TILE + r, n = J * TILE + c0 + c;
            win[h * TILE + r][c] = (m < nbf && n < nbf) ? v : 0.0;
        }
    }
    if (threadIdx.x < MM) {
        const int m = mb * MM + threadIdx.x;
        const int E = exp_of_max_d(rowmax[(size_t)Q * nbf_p + m]);
        Es[threadIdx.x] = E;
        if (b == mb_ptr[mb]) sA[(size_t)Q * nbf_p + m] = scale_of(E);
    }
    __syncthreads();
    uint8_t* out = Bd + id * I8_BLOCK;
    for (int u = threadIdx.x; u < MM * (MK / 8); u += blockDim.x) {
        const int r = u / (MK / 8), c8 = (u % (MK / 8)) * 8;
        const int E = Es[r];
        uint32_t w[NSL][2];
#pragma unroll
        for (int s = 0; s < NSL; ++s) w[s][0] = w[s][1] = 0u;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const unsigned long long uu = (unsigned long long)(fix_d(win[r][c8 + j], E) + (long long)DIGIT_OFF);
#pragma unroll
            for (int s = 0; s < NSL; ++s) w[s][j / 4] |= digit_field(uu, s) << (8 * (j % 4));
        }
#pragma unroll
        for (int s = 0; s < NSL; ++s)
            *reinterpret_cast<uint2*>(out + s * I8_SLICE + r * MK + c8) = make_uint2(w[s][0], w[s][1]);
    }
}

// ---------------------------------------------------------------- digits of C (every build)
// Column exponents of C (nbf x nocc_pad, row-major): one block per column slot i < ncols.
__global__ void oz_col_scale_kernel(const double* __restrict__ C, int nbf, int nocc_pad, int nocc,
                                    int* __restrict__ eC, float* __restrict__ sC, int* __restrict__ err) {
    const int i = blockIdx.x;
    unsigned long long mx = 0;
    if (i < nocc)
        for (int n = threadIdx.x; n < nbf; n += blockDim.x) {
            unsigned long long b = (unsigned long long)__double_as_longlong(C[(size_t)n * nocc_pad + i]) &
                                   0x7FFFFFFFFFFFFFFFull;
            mx = b > mx ? b : mx;
        }
    __shared__ unsigned long long red[32];
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x / 32] = mx;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long m2 = 0;
        for (int w = 0; w < (int)(blockDim.x / 32); ++w) m2 = max(m2, red[w]);
        const int E = exp_of_max_d(m2);
        eC[i] = E;
        sC[i] = scale_of(E);
        if (m2 >= NONFINITE_BITS) atomicOr(err, DEV_ERR_NUMERIC);
    }
}

// BF16 digit slices of C^T for the half-transform's B operand: [chunk][kb][slice][N rows][32 k],
// each (N x 32) slice pre-swizzled (64-byte rows).  Thread = (column slot i, 8 consecutive n).
__global__ void oz_split_C_kernel(const double* __restrict__ C, int nbf, int nbf_p, int nocc_pad, int N, int ncols,
                                  const int* __restrict__ eC, __nv_bfloat16* __restrict__ Cd) {
    const int n8 = nbf_p / 8;
    const size_t total = (size_t)ncols * n8;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < total; e += (size_t)gridDim.x * blockDim.x) {
        const int i = (int)(e / n8), n0 = (int)(e % n8) * 8;
        const int E = eC[i];
        uint32_t w[NSL][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int n = n0 + j;
            const double x = (n < nbf && i < nocc_pad) ? C[(size_t)n * nocc_pad + i] : 0.0;
            const unsigned long long uu = (unsigned long long)(fix_d(x, E) + (long long)DIGIT_OFF);
#pragma unroll
            for (int s = 0; s < NSL; ++s) {
                const uint32_t bits = field_bf16(digit_field(uu, s), slice_weight(s));
                if (j % 2 == 0)
                    w[s][j / 2] = bits;
                else
                    w[s][j / 2] |= bits << 16;
            }
        }
        const int chunk = i / N, row = i % N, kb = n0 / MK, c = (n0 % MK) / 8;
        const int nkb = nbf_p / MK;
        __nv_bfloat16* base = Cd + ((size_t)chunk * nkb + kb) * NSL * N * MK;
        const uint32_t off = tc::swz_offset((uint32_t)row, (uint32_t)c) / 2;
#pragma unroll
        for (int s = 0; s < NSL; ++s)
            *reinterpret_cast<uint4*>(base + (size_t)s * N * MK + off) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
}

// ---------------------------------------------------------------- shared pieces of the GEMMs
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
    s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// a[0] + ... + a[5] as an unevaluated FP32 pair (hi, lo): a[0..4] are the exact level sums,
// a[5] the small tail; TwoSums and a final Fast2Sum keep the error near 2^-45 |hi|.
__device__ __forceinline__ void combine6(const float* a, float& hi, float& lo) {
    float s, e1, e2, e3, e4;
    two_sum(a[0], a[1], s, e1);
    two_sum(s, a[2], s, e2);
    two_sum(s, a[3], s, e3);
    two_sum(s, a[4], s, e4);
    const float l = __fadd_rn(__fadd_rn(__fadd_rn(e1, e2), __fadd_rn(e3, e4)), a[5]);
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

// (H, L) += (hi, lo), double-float
__device__ __forceinline__ void df_add(float& H, float& L, float hi, float lo) {
    float s, e;
    two_sum(H, hi, s, e);
    const float l = __fadd_rn(L, __fadd_rn(e, lo));
    H = __fadd_rn(s, l);
    L = __fsub_rn(l, __fsub_rn(H, s));
}

// ---------------------------------------------------------------- half-transform
struct TrArgs {
    const uint8_t* Bd;         // int8 digit fields of B, [Q][mb][kb][7][128][32]
    const __nv_bfloat16* Cd;   // BF16 digit slices of C^T, [chunk][kb][7][N][32]
    const float* sA;           // [Q][nbf_p] slice weight 2^(E-5) of each row of B
    const float* sC;           // [nchunk * N] slice weight of each column of C
    float2* Xdf;               // [nbf][kdim_b] X as (hi, lo), k = (Q - q0) * nocc_p + i
    unsigned* xmax;            // [nbf][ngroups] max |hi| per (row, group of G aux functions)
    int q0, nq, nmb, nkb, nbf, nbf_p, nocc_p, N, nchunk, G, ngroups;
    const int* mb_ptr;         // listed k blocks of row block mb: mb_kb[mb_ptr[mb] .. mb_ptr[mb+1])
    const int* mb_kb;
    int nnz;                   // listed blocks in all (the digit blocks of one Q)
    int run_kb;                // listed k blocks per accumulation run, at most
    size_t kdim_b;
    int stages, nbuf, n_items, ncols;
    int* err;
    // extents of the buffers (checked in the bounds-checked build): Bd in bytes, the rest in
    // elements
    size_t lim_Bd, lim_Cd, lim_X, lim_xmax, lim_sA;
};

// The half-transform keeps its A operand (the digit slices of B) in tensor memory: the
// converter warps write each converted slice straight into one of TR_ASLOTS 16-column TMEM
// slots with tcgen05.st, and the MMAs read A from there (only C^T comes from shared memory).
// Its accumulators: levels 0-3 exact and a tail (4-6); the round-toward-zero truncation of
// the tail is harmless here (no sums of squares; it is random relative to X).
constexpr int TR_NACC = 5;
constexpr int TR_ASLOTS = 7;  // a whole k block of A slices: the converters run one k block ahead
static_assert(TR_ASLOTS == NSL, "slot r holds slice r of every k block (the slot pairs follow the slice pairs)");
constexpr int TR_ACOL0 = 512 - TR_ASLOTS * 16;  // first A-slot column
constexpr int TR_OFF_C = NSL * I8_SLICE;        // stage: [7 int8 A slices | 7 BF16 C^T slices]

__device__ __forceinline__ void tr_item(const TrArgs& a, int item, int& Q, int& mb, int& chunk) {
    chunk = item % a.nchunk;
    const int rest = item / a.nchunk;
    mb = rest % a.nmb;
    Q = a.q0 + rest / a.nmb;
}
// the listed k blocks of row block mb: first list position, count, runs, positions per run
__device__ __forceinline__ void tr_blocks(const TrArgs& a, int mb, int& p0, int& cnt, int& nrun, int& rlen) {
    p0 = a.mb_ptr[mb];
    cnt = a.mb_ptr[mb + 1] - p0;
    nrun = max(1, (cnt + a.run_kb - 1) / a.run_kb);
    rlen = (cnt + nrun - 1) / nrun;
}

// a[0] + ... + a[4]: four exact level sums and the tail, as an FP32 pair
__device__ __forceinline__ void combine5(const float* a, float& hi, float& lo) {
    float s, e1, e2, e3;
    two_sum(a[0], a[1], s, e1);
    two_sum(s, a[2], s, e2);
    two_sum(s, a[3], s, e3);
    const float l = __fadd_rn(__fadd_rn(__fadd_rn(e1, e2), e3), a[4]);
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

// MMA with the A operand in tensor memory
__device__ __forceinline__ void mma_bf16_ta(uint32_t d_tmem, uint32_t a_tmem, uint64_t bdesc, uint32_t idesc,
                                            uint32_t accum) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p;\n\t}" ::"r"(d_tmem),
        "r"(a_tmem), "l"(bdesc), "r"(idesc), "r"(accum)
        : "memory");
}
__device__ __forceinline__ void tmem_st16(uint32_t taddr, const uint32_t* v) {
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};" ::"r"(
            taddr),
        "r"(v[0]), "r"(v[1]), "r"(v[2]), "r"(v[3]), "r"(v[4]), "r"(v[5]), "r"(v[6]), "r"(v[7]), "r"(v[8]), "r"(v[9]),
        "r"(v[10]), "r"(v[11]), "r"(v[12]), "r"(v[13]), "r"(v[14]), "r"(v[15])
        : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// one A slice (slot at TMEM column a_col) against the C^T slices of the stage: pairs (J, t),
// t <= 6 - J, into accumulator min(J + t, 4); `first` starts a fresh accumulation run.
// PART 0 issues the pairs of the exact levels (accumulators 0..NA-2), PART 1 those of the tail
// (accumulator NA-1): two threads issue them, each accumulator has one issuer, so the order of
// the MMAs into an accumulator is the same as from a single issuer.
template <int NA, int J, int PART>
__device__ __forceinline__ void issue_slice(const uint32_t* d, uint32_t a_col, uint64_t dB, uint64_t b_step, uint32_t id,
                                            bool first) {
#pragma unroll
    for (int ks = 0; ks < MK / 16; ++ks) {
#pragma unroll
        for (int t = 0; t <= NSL - 1 - J; ++t) {
            const int L = J + t < NA - 1 ? J + t : NA - 1;
            if ((L < NA - 1) != (PART == 0)) continue;
            const uint32_t f = (first && ks == 0 && J == 0 && t <= NA - 1) ? 0u : 1u;
            mma_bf16_ta(d[L], a_col + (uint32_t)(8 * ks), dB + (uint64_t)t * b_step + (uint64_t)(2 * ks), id, f);
        }
    }
}

// slice j (0..6) of the A operand from its TMEM slot: of the (7 - j) pairs with B slices
// 0..6-j, those of issuer PART
template <int NA, int PART>
__device__ __forceinline__ void issue_slice_j(int j, const uint32_t* d, uint32_t a_col, uint64_t dB, uint64_t b_step,
                                              uint32_t id, bool first) {
    switch (j) {
        case 0: issue_slice<NA, 0, PART>(d, a_col, dB, b_step, id, first); break;
        case 1: issue_slice<NA, 1, PART>(d, a_col, dB, b_step, id, first); break;
        case 2: issue_slice<NA, 2, PART>(d, a_col, dB, b_step, id, first); break;
        case 3: issue_slice<NA, 3, PART>(d, a_col, dB, b_step, id, first); break;
        case 4: issue_slice<NA, 4, PART>(d, a_col, dB, b_step, id, first); break;
        case 5: issue_slice<NA, 5, PART>(d, a_col, dB, b_step, id, first); break;
        default: issue_slice<NA, 6, PART>(d, a_col, dB, b_step, id, first); break;
    }
}

// The contraction's MMAs with NS digits and levels up to MAXL: A slice J (shared-memory
// descriptor dA; 16 k = 2 descriptor units) against B slices t <= min(NS - 1, MAXL - J).  The
// exact level regions d[0..NA-2] lie side by side in TMEM (CT_N columns each) and the B slices
// one after another in the stage (slice t at row t*CT_N), so the pairs of levels J..NA-2 are
// one operand of NW*CT_N rows, issued as MMAs of up to 256 columns; the tail pairs (level
// >= NA-1) follow one by one into d[NA-1].
template <int NS, int NA, int MAXL, int J>
__device__ __forceinline__ void issue_slice_gs(const uint32_t* d, uint64_t dA, uint64_t dB, uint64_t b_step, uint32_t id,
                                               bool first) {
    constexpr int TMAX = (NS - 1) < (MAXL - J) ? (NS - 1) : (MAXL - J);
    constexpr int NW0 = NA - 1 - J < 0 ? 0 : NA - 1 - J;
    constexpr int NW = NW0 < TMAX + 1 ? NW0 : TMAX + 1;  // B slices of the wide operand
    constexpr int ROWS = NW * CT_N;
    const uint32_t id0 = id & ~(0x3Fu << 17);
#pragma unroll
    for (int ks = 0; ks < MK / 16; ++ks) {
        const uint32_t fw = (first && ks == 0 && J == 0) ? 0u : 1u;
#pragma unroll
        for (int r0 = 0; r0 < ROWS; r0 += 256) {
            const int n = ROWS - r0 < 256 ? ROWS - r0 : 256;
            tc::mma_bf16(d[J] + (uint32_t)r0, dA + (uint64_t)(2 * ks), dB + (uint64_t)(r0 * 4 + 2 * ks),
                         id0 | ((uint32_t)(n >> 3) << 17), fw);
        }
#pragma unroll
        for (int t = NW; t <= TMAX; ++t) {
            const uint32_t f = (first && ks == 0 && J == 0 && t == NA - 1) ? 0u : 1u;
            tc::mma_bf16(d[NA - 1], dA + (uint64_t)(2 * ks), dB + (uint64_t)t * b_step + (uint64_t)(2 * ks), id, f);
        }
    }
}
template <int NS, int NA, int MAXL>
__device__ __forceinline__ void issue_slice_gjs(int j, const uint32_t* d, uint64_t dA, uint64_t dB, uint64_t b_step,
                                                uint32_t id, bool first) {
    switch (j) {
        case 0: issue_slice_gs<NS, NA, MAXL, 0>(d, dA, dB, b_step, id, first); break;
        case 1: issue_slice_gs<NS, NA, MAXL, 1>(d, dA, dB, b_step, id, first); break;
        case 2: issue_slice_gs<NS, NA, MAXL, 2>(d, dA, dB, b_step, id, first); break;
        case 3: issue_slice_gs<NS, NA, MAXL, 3>(d, dA, dB, b_step, id, first); break;
        case 4: issue_slice_gs<NS, NA, MAXL, 4>(d, dA, dB, b_step, id, first); break;
        case 5: issue_slice_gs<NS, NA, MAXL, 5>(d, dA, dB, b_step, id, first); break;
        case 6: issue_slice_gs<NS, NA, MAXL, 6>(d, dA, dB, b_step, id, first); break;
        default: issue_slice_gs<NS, NA, MAXL, (NS > 7 ? 7 : 6)>(d, dA, dB, b_step, id, first); break;
    }
}

// a[0] + ... + a[NA-1]: NA - 1 exact level sums and the tail, as an FP32 pair
template <int NA>
__device__ __forceinline__ void combine_n(const float* a, float& hi, float& lo) {
    float s = a[0], l = 0.f;
#pragma unroll
    for (int i = 1; i < NA - 1; ++i) {
        float e;
        two_sum(s, a[i], s, e);
        l = __fadd_rn(l, e);
    }
    l = __fadd_rn(l, a[NA - 1]);
    hi = __fadd_rn(s, l);
    lo = __fsub_rn(l, __fsub_rn(hi, s));
}

// Persistent, warp-specialised: warp 0 lane 0 bulk-copies one k block (int8 A + BF16 C^T) per
// stage; warps 6-9 convert A slice by slice into TMEM slots (each thread its own row);
// warp 1 lane 0 issues the slice-pair MMAs of the exact levels and warp 14 lane 0 those of the
// tail (one thread issuing all 56 MMAs of a k block was the limit: ~89 cycles per MMA against
// ~39 of tensor work); warps 2-5 and 10-13 drain the accumulators (tcgen05.ld) after every run
// into double-float X and take the row maxima.
__global__ void __launch_bounds__(TR_THREADS, 1) oz_transform_kernel(const TrArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int N = a.N;
    const int c_slice = N * MK * 2;
    const int stage_bytes = TR_OFF_C + NSL * c_slice;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)a.stages * stage_bytes);
    uint64_t* empty = full + a.stages;
    uint64_t* afull = empty + a.stages;   // [TR_ASLOTS]
    uint64_t* aempty = afull + TR_ASLOTS; // [TR_ASLOTS]
    uint64_t* tfull = aempty + TR_ASLOTS; // [2]
    uint64_t* tempty = tfull + 2;         // [2]
    uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(tempty + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);
    float* s_sc = reinterpret_cast<float*>(tmem_holder + 4);  // slice weights of the columns of C
    const int warp = threadIdx.x / 32;
    for (int i = threadIdx.x; i < a.ncols; i += blockDim.x) s_sc[i] = a.sC[i];
    if (threadIdx.x == 0) {
        for (int s = 0; s < a.stages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 2);  // both MMA issuers commit
        }
        for (int r = 0; r < TR_ASLOTS; ++r) {
            tc::mbar_init(&afull[r], 128);
            tc::mbar_init(&aempty[r], 2);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tfull[b], 2);
            tc::mbar_init(&tempty[b], 8);
        }
        *abort_flag = 0;
        tc::fence_barrier_init();
    }
    if (warp == 0) tc::tmem_alloc(tmem_holder, 512u);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;

    if (threadIdx.x == 0) {
        // ---- producer: one stage per k block
        int s = 0;
        uint32_t ph = 0;
        long kg = 0;
        bool ok = true;
        const uint32_t cbytes = (uint32_t)(NSL * c_slice);
        for (int item = blockIdx.x; ok && item < a.n_items && !*abort_flag; item += gridDim.x) {
            int Q, mb, chunk;
            tr_item(a, item, Q, mb, chunk);
            int p0, cnt, nrun, rlen;
            tr_blocks(a, mb, p0, cnt, nrun, rlen);
            const uint8_t* pa = a.Bd + ((size_t)Q * a.nnz + p0) * I8_BLOCK;
            const __nv_bfloat16* pc = a.Cd + (size_t)chunk * a.nkb * NSL * N * MK;
            for (int p = 0; p < cnt; ++p, ++kg) {
                if (kg >= a.stages && !tc::mbar_wait(&empty[s], ph ^ 1u, abort_flag, a.err)) {
                    ok = false;
                    break;
                }
                if (!BCHK(p0 + p < a.nnz, a.err, BC_TR_LIST, p0 + p, a.nnz) ||
                    !BRANGE(((size_t)Q * a.nnz + p0 + p) * I8_BLOCK, I8_BLOCK, a.lim_Bd, a.err, BC_TR_BD) ||
                    !BRANGE(((size_t)chunk * a.nkb + a.mb_kb[p0 + p]) * NSL * N * MK, (size_t)NSL * N * MK, a.lim_Cd,
                            a.err, BC_TR_CD)) {
                    *abort_flag = 1;  // the consumers leave their waits; no copy of this stage was issued
                    ok = false;
                    break;
                }
                uint8_t* st = smem + (size_t)s * stage_bytes;
                tc::mbar_arrive_expect_tx(&full[s], (uint32_t)I8_BLOCK + cbytes);
                tc::bulk_load(st, pa + (size_t)p * I8_BLOCK, (uint32_t)I8_BLOCK, &full[s]);
                tc::bulk_load(st + TR_OFF_C, pc + (size_t)a.mb_kb[p0 + p] * NSL * N * MK, cbytes, &full[s]);
                if (++s == a.stages) {
                    s = 0;
                    ph ^= 1u;
                }
            }
        }
    } else if (warp >= 6 && warp < 10) {
        // ---- converters: row `row` of every slice, int8 field f = d + 64 in [0, 127] -> BF16
        // d * 2^(-7 slice), two K elements per 32-bit TMEM column, into the next A slots, two
        // slices per step.  A byte permute puts f under the BF16 exponent of 128 (bits
        // 0x4300 | f are the value 128 + f = 192 + d, exactly), and one BF16x2 FMA gives
        // (192 + d) w - 192 w = d w exactly: two instructions per two elements.
        const int q = warp % 4;
        const int row = q * 32 + (threadIdx.x % 32);
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
        int s = 0, r = 0;
        uint32_t ph = 0, pr = 0;
        long used = 0;
        bool ok = true;
        for (int item = blockIdx.x; ok && item < a.n_items; item += gridDim.x) {
            int Q, mb, chunk, p0, cnt, nrun, rlen;
            tr_item(a, item, Q, mb, chunk);
            tr_blocks(a, mb, p0, cnt, nrun, rlen);
            for (int p = 0; ok && p < cnt; ++p) {
                if (!tc::mbar_wait(&full[s], ph, abort_flag, a.err)) {
                    ok = false;
                    break;
                }
                const uint8_t* st = smem + (size_t)s * stage_bytes;
#pragma unroll 1
                for (int j0 = 0; ok && j0 < NSL; j0 += 2) {
                    const int nj = NSL - j0 < 2 ? NSL - j0 : 2;
                    int slot[2] = {0, 0};
                    for (int jj = 0; jj < nj; ++jj, ++used) {
                        // the issuers release a pair of slots with one commit on its last slot
                        if (jj == nj - 1 && used >= TR_ASLOTS &&
                            !tc::mbar_wait(&aempty[r], pr ^ 1u, abort_flag, a.err)) {
                            ok = false;
                            break;
                        }
                        slot[jj] = r;
                        if (++r == TR_ASLOTS) {
                            r = 0;
                            pr ^= 1u;
                        }
                    }
                    if (!ok) break;
                    tc::tc_fence_after();
                    for (int jj = 0; jj < nj; ++jj) {
                        const int j = j0 + jj;
                        const uint4 q0 = *reinterpret_cast<const uint4*>(st + j * I8_SLICE + row * MK);
                        const uint4 q1 = *reinterpret_cast<const uint4*>(st + j * I8_SLICE + row * MK + 16);
                        const uint32_t words[8] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y, q1.z, q1.w};
                        const float w = slice_weight(j);
                        const __nv_bfloat162 wv = __float2bfloat162_rn(w);            // 2^(-7j), exact
                        const __nv_bfloat162 cv = __float2bfloat162_rn(-192.0f * w);  // exact
                        uint32_t o[16];
#pragma unroll
                        for (int wi = 0; wi < 8; ++wi) {
#pragma unroll
                            for (int hh = 0; hh < 2; ++hh) {
                                // bytes (f_{2hh}, 0x43, f_{2hh+1}, 0x43): low half the even k
                                const uint32_t x = __byte_perm(words[wi], 0x43434343u, hh ? 0x5342u : 0x5140u);
                                const __nv_bfloat162 g = __hfma2(*reinterpret_cast<const __nv_bfloat162*>(&x), wv, cv);
                                o[2 * wi + hh] = *reinterpret_cast<const uint32_t*>(&g);
                            }
                        }
                        tmem_st16(lane_base + (uint32_t)(TR_ACOL0 + 16 * slot[jj]), o);
                    }
                    tmem_wait_st();
                    tc::tc_fence_before();
                    // one arrival for the pair, on its last slot: every thread's stores to both
                    // slots completed before it
                    tc::mbar_arrive(&afull[nj == 2 ? slot[1] : slot[0]]);
                }
                if (++s == a.stages) {
                    s = 0;
                    ph ^= 1u;
                }
            }
        }
    } else if (threadIdx.x == 32 || threadIdx.x == 448) {
        // ---- MMA issuers (warp 1: the exact levels' pairs, warp 14: the tail's): per k block,
        // seven A slices from TMEM slots against one stage; both wait for every stage and A
        // slot and both commit every release (the barriers count two arrivals)
        const bool tail = threadIdx.x == 448;
        int s = 0, r = 0;
        uint32_t ph = 0, pr = 0;
        int ri = 0;
        const uint32_t smem_base = tc::smem_u32(smem);
        const uint32_t id = tc::idesc_bf16_f32(MM, N, false);
        const uint64_t b_step = (uint64_t)(c_slice >> 4);
        bool ok = true;
        for (int item = blockIdx.x; ok && item < a.n_items && !*abort_flag; item += gridDim.x) {
            int Q, mb, chunk, p0, cnt, nrun, rlen;
            tr_item(a, item, Q, mb, chunk);
            tr_blocks(a, mb, p0, cnt, nrun, rlen);
            for (int run = 0; ok && run < nrun; ++run, ++ri) {
                const int buf = ri % a.nbuf, use = ri / a.nbuf;
                if (use > 0 && !tc::mbar_wait(&tempty[buf], (uint32_t)((use - 1) & 1), abort_flag, a.err)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t d0 = tmem + (uint32_t)(buf * TR_NACC * N);
                uint32_t d[TR_NACC];
#pragma unroll
                for (int L = 0; L < TR_NACC; ++L) d[L] = d0 + (uint32_t)(L * N);
                const int kb0 = run * rlen, kb1 = min(cnt, kb0 + rlen);  // list positions of this run
                for (int kb = kb0; ok && kb < kb1; ++kb) {
                    if (!tc::mbar_wait(&full[s], ph, abort_flag, a.err)) {
                        ok = false;
                        break;
                    }
                    const uint64_t dB = tc::sdesc_kmajor(smem_base + (uint32_t)(s * stage_bytes + TR_OFF_C));
                    const bool first = kb == kb0;
#pragma unroll
                    for (int j = 0; j < NSL; ++j) {
                        // the converters fill slots in pairs (j, j + 1) and arrive on the pair's
                        // last slot only (each k block uses all seven slots, so r == j here):
                        // one poll and one commit per pair
                        const bool pair_first = (j & 1) == 0;
                        const bool pair_last = (j & 1) == 1 || j == NSL - 1;
                        if (pair_first) {
                            const int rl = j + 1 < NSL ? r + 1 : r;
                            if (!tc::mbar_wait(&afull[rl], pr, abort_flag, a.err)) {
                                ok = false;
                                break;
                            }
                            tc::tc_fence_after();
                        }
                        const uint32_t a_col = tmem + (uint32_t)(TR_ACOL0 + 16 * r);
                        if (tail)
                            issue_slice_j<TR_NACC, 1>(j, d, a_col, dB, b_step, id, first);
                        else
                            issue_slice_j<TR_NACC, 0>(j, d, a_col, dB, b_step, id, first);
                        if (pair_last) tc::mma_commit(&aempty[r]);
                        if (++r == TR_ASLOTS) {
                            r = 0;
                            pr ^= 1u;
                        }
                    }
                    if (!ok) break;
                    tc::mma_commit(&empty[s]);
                    if (++s == a.stages) {
                        s = 0;
                        ph ^= 1u;
                    }
                }
                tc::mma_commit(&tfull[buf]);
            }
        }
    } else if (warp >= 2 && warp < 14) {
        // ---- epilogue (warps 2-5 and 10-13, one column half each): after each run,
        // X (+)= run sum; after the last, the row maximum
        const int q = warp % 4;
        const int half = warp >= 10 ? 1 : 0;
        const int rr = q * 32 + (threadIdx.x % 32);
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
        int ri = 0;
        bool ok = true;
        for (int item = blockIdx.x; ok && item < a.n_items; item += gridDim.x) {
            int Q, mb, chunk;
            tr_item(a, item, Q, mb, chunk);
            const int m = mb * MM + rr;
            bool valid = m < a.nbf;
            // the row's weight and its nocc_p elements of X (read back after the first run)
            if (valid && (!BCHK((size_t)Q * a.nbf_p + m < a.lim_sA, a.err, BC_TR_SA, (size_t)Q * a.nbf_p + m, a.lim_sA) ||
                          !BRANGE((size_t)m * a.kdim_b + (size_t)(Q - a.q0) * a.nocc_p, a.nocc_p, a.lim_X, a.err,
                                  BC_TR_X)))
                valid = false;
            const float sa = valid ? a.sA[(size_t)Q * a.nbf_p + m] : 0.f;
            float2* xrow = a.Xdf + (valid ? (size_t)m * a.kdim_b + (size_t)(Q - a.q0) * a.nocc_p : 0);
            float rmax = 0.f;
            int p0, cnt, nrun, rlen;
            tr_blocks(a, mb, p0, cnt, nrun, rlen);
            for (int run = 0; run < nrun; ++run, ++ri) {
                const int buf = ri % a.nbuf, use = ri / a.nbuf;
                ok = tc::mbar_wait(&tfull[buf], (uint32_t)(use & 1), abort_flag, a.err);
                __syncwarp();
                if (!ok || *abort_flag) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t cb = lane_base + (uint32_t)(buf * TR_NACC * N);
                const bool last = run == nrun - 1;
                for (int c0 = half * (N / 2); c0 < (half + 1) * (N / 2); c0 += 8) {
                    const int i0 = chunk * N + c0;
                    float2 prev[8];
                    if (run > 0 && valid) {
#pragma unroll
                        for (int j = 0; j < 8; ++j) prev[j] = i0 + j < a.nocc_p ? xrow[i0 + j] : make_float2(0.f, 0.f);
                    }
                    uint32_t v[TR_NACC][8];
#pragma unroll
                    for (int L = 0; L < TR_NACC; ++L) tc::tmem_ld8_nowait(cb + (uint32_t)(L * N + c0), v[L]);
                    tc::tmem_wait_ld();
                    if (valid) {
#pragma unroll
                        for (int j = 0; j < 8; ++j) {
                            const int i = i0 + j;
                            if (i < a.nocc_p) {
                                float acc[TR_NACC];
#pragma unroll
                                for (int L = 0; L < TR_NACC; ++L) acc[L] = __uint_as_float(v[L][j]);
                                float hi, lo;
                                combine5(acc, hi, lo);
                                const float sc = sa * s_sc[i];
                                hi *= sc;
                                lo *= sc;
                                if (run > 0) {
                                    float H = prev[j].x, Lo = prev[j].y;
                                    df_add(H, Lo, hi, lo);
                                    hi = H;
                                    lo = Lo;
                                }
                                xrow[i] = make_float2(hi, lo);
                                if (last) rmax = fmaxf(rmax, fabsf(hi));
                            }
                        }
                    }
                }
                tc::tc_fence_before();
                __syncwarp();
                if ((threadIdx.x % 32) == 0) tc::mbar_arrive(&tempty[buf]);
            }
            if (ok && valid && rmax > 0.f &&
                BCHK((size_t)m * a.ngroups + (Q - a.q0) / a.G < a.lim_xmax, a.err, BC_TR_XMAX,
                     (size_t)m * a.ngroups + (Q - a.q0) / a.G, a.lim_xmax))
                atomicMax(&a.xmax[(size_t)m * a.ngroups + (Q - a.q0) / a.G], __float_as_uint(rmax));
        }
    }
    __syncwarp();
    if (*abort_flag && threadIdx.x == 0) {
        // let copies already issued land before the block's shared memory goes away
        uint64_t t0 = tc::global_timer();
        while (tc::global_timer() - t0 < 10000000ull) {
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 512u);
}

// ---------------------------------------------------------------- split of X
// X (double-float) -> BF16 digit slices for the contraction, [mb][kbt][7][128][32] pre-swizzled,
// one exponent per (row, group); also the slice weights Sx[g][m] = 2^(E-5).
// Block = (128-row block, group); 256 threads, thread unit = (row, 8 consecutive k).
__global__ void __launch_bounds__(256) oz_split_X_kernel(const float2* __restrict__ Xdf, const unsigned* __restrict__ xmax,
                                                         int nbf, int nbf_p, int ngroups, int G, int nq, int nocc_p,
                                                         size_t kdim_b, size_t nkbt, float* __restrict__ Sx,
                                                         __nv_bfloat16* __restrict__ Xd, size_t lim_X, size_t lim_Xd,
                                                         size_t lim_Sx, int* __restrict__ err) {
    const int mb = blockIdx.x, g = blockIdx.y;
    __shared__ int Es[MM];
    if (threadIdx.x < MM) {
        const int m = mb * MM + threadIdx.x;
        int E = m < nbf ? exp_of_max_f(xmax[(size_t)m * ngroups + g]) : E_EMPTY;
        // the row's X elements of this group
        const size_t kb0 = (size_t)g * G * nocc_p / MK, kb1 = (size_t)min(nq, (g + 1) * G) * nocc_p / MK;
        if (E != E_EMPTY && !BRANGE((size_t)m * kdim_b + kb0 * MK, (kb1 - kb0) * MK, lim_X, err, BC_SX_READ))
            E = E_EMPTY;
        Es[threadIdx.x] = E;
        if (BCHK((size_t)g * nbf_p + m < lim_Sx, err, BC_SX_SX, (size_t)g * nbf_p + m, lim_Sx))
            Sx[(size_t)g * nbf_p + m] = scale_of(E);
    }
    __syncthreads();
    const int kb0 = g * G * nocc_p / MK;
    const int kb1 = min(nq, (g + 1) * G) * nocc_p / MK;
    const int units = (kb1 - kb0) * MM * (MK / 8);
    for (int u = threadIdx.x; u < units; u += blockDim.x) {
        const int kb = kb0 + u / (MM * (MK / 8));
        const int rem = u % (MM * (MK / 8));
        const int r = rem / (MK / 8), c = rem % (MK / 8);
        const int m = mb * MM + r;
        const int E = Es[r];
        uint32_t w[NSL][4];
#pragma unroll
        for (int s = 0; s < NSL; ++s) w[s][0] = w[s][1] = w[s][2] = w[s][3] = 0u;
        if (E != E_EMPTY) {
            const float4* src = reinterpret_cast<const float4*>(Xdf + (size_t)m * kdim_b + (size_t)kb * MK + c * 8);
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const float4 x = src[p];  // two (hi, lo) pairs
                const unsigned long long u0 = (unsigned long long)(fix_f(x.x, E) + fix_f(x.y, E) + (long long)DIGIT_OFF);
                const unsigned long long u1 = (unsigned long long)(fix_f(x.z, E) + fix_f(x.w, E) + (long long)DIGIT_OFF);
#pragma unroll
                for (int s = 0; s < NSL; ++s) {
                    const float wt = slice_weight(s);
                    w[s][p] = field_bf16(digit_field(u0, s), wt) | (field_bf16(digit_field(u1, s), wt) << 16);
                }
            }
        }
        __nv_bfloat16* base = Xd + ((size_t)mb * nkbt + kb) * NSL * (MM * MK);
        const uint32_t off = tc::swz_offset((uint32_t)r, (uint32_t)c) / 2;
        if (!BRANGE(((size_t)mb * nkbt + kb) * NSL * (MM * MK), (size_t)NSL * MM * MK, lim_Xd, err, BC_SX_WRITE)) continue;
#pragma unroll
        for (int s = 0; s < NSL; ++s)
            *reinterpret_cast<uint4*>(base + (size_t)s * (MM * MK) + off) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
    }
}

// ---------------------------------------------------------------- contraction
struct CtArgs {
    const __nv_bfloat16* Xd;  // row operand digits [mb][kbt][7][128][32]
    const __nv_bfloat16* Yd;  // column operand digits, same layout (= Xd for K = X X^T)
    const float* Sx;          // row weights [group][lds_x]
    const float* Sy;          // column weights [group][lds_y]
    const int2* tiles;        // (128-row block, 64-column block): the lower triangle for K
    int ntiles, nsplit, gps, ngroups;
    int kpg, nkb;             // k blocks per group (one accumulation run), k blocks in all
    int lds_x, lds_y;
    size_t nkbt;              // k-block stride of the digit arrays
    double* part;             // [nsplit][ntiles][128][64] (out == nullptr)
    double* out;              // general product: out[m][n] (+)= result for m < M, n < N
    size_t ldo;
    int M, N, accumulate;
    int stages, n_items;
    int* err;
    // extents in elements (checked in the bounds-checked build); lim_out covers part or out
    size_t lim_Xd, lim_Yd, lim_Sx, lim_Sy, lim_out;
};

// Stage per k block: [NS A slices, 128 rows | NS B slices, 64 rows], both read by the MMAs
// straight from shared memory (64-byte swizzled, K-major).  K = X X^T: 7 digits, six
// accumulators (levels 0-4 exact, tail 5-6) at TMEM columns 0..383.  The general product
// (metric contraction): 8 digits, levels <= 8, seven accumulators (levels 0-5 exact, tail 6-8)
// at 0..447.
constexpr int CT_NACC = NACC;
constexpr int CT_THREADS = 320;  // producer, MMA, 8 epilogue warps
__host__ __device__ constexpr int ct_stage_bytes(int ns) { return ns * BF_SLICE + ns * CT_N * MK * 2; }
constexpr int CT_STAGE = ct_stage_bytes(NSL);  // 84 KB
constexpr int GM_NS = 8, GM_NACC = 7, GM_MAXL = 8;
static_assert(GM_NACC * CT_N <= 512 && CT_NACC * CT_N <= 512, "TMEM columns");

__device__ __forceinline__ void ct_item(const CtArgs& a, int item, int& tile, int& g0, int& g1) {
    const int split = item / a.ntiles;  // split-major: concurrent CTAs share one k window in L2
    tile = item % a.ntiles;
    g0 = split * a.gps;
    g1 = min(a.ngroups, g0 + a.gps);
}
__device__ __forceinline__ int ct_kb0(const CtArgs& a, int g) { return g * a.kpg; }
__device__ __forceinline__ int ct_kb1(const CtArgs& a, int g) { return min(a.nkb, (g + 1) * a.kpg); }

template <int NS, int NA, int MAXL, bool DIRECT>
__global__ void __launch_bounds__(CT_THREADS, 1) oz_contract_kernel(const CtArgs a) {
    constexpr int OFF_B = NS * BF_SLICE;
    constexpr int STAGE = ct_stage_bytes(NS);
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)a.stages * STAGE);
    uint64_t* empty = full + a.stages;
    uint64_t* tfull = empty + a.stages;  // [2]
    uint64_t* tempty = tfull + 2;        // [2]
    uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(tempty + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);
    const int warp = threadIdx.x / 32;
    if (threadIdx.x == 0) {
        for (int s = 0; s < a.stages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tfull[b], 1);
            tc::mbar_init(&tempty[b], 8);
        }
        *abort_flag = 0;
        tc::fence_barrier_init();
    }
    if (warp == 0) tc::tmem_alloc(tmem_holder, 512u);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;
    const size_t blk = (size_t)MM * MK;  // elements of one slice block

    if (threadIdx.x == 0) {
        // ---- producer: one stage per k block
        int s = 0;
        uint32_t ph = 0;
        long kg = 0;
        bool ok = true;
        for (int item = blockIdx.x; ok && item < a.n_items && !*abort_flag; item += gridDim.x) {
            int tile, g0, g1;
            ct_item(a, item, tile, g0, g1);
            const int2 tb = a.tiles[tile];
            const __nv_bfloat16* pa = a.Xd + (size_t)tb.x * a.nkbt * NS * blk;
            const __nv_bfloat16* pb = a.Yd + (size_t)(tb.y / 2) * a.nkbt * NS * blk + (size_t)(tb.y % 2) * (CT_N * MK);
            for (int g = g0; ok && g < g1; ++g) {
                const int kb0 = ct_kb0(a, g), kb1 = ct_kb1(a, g);
                for (int kb = kb0; kb < kb1; ++kb, ++kg) {
                    if (kg >= a.stages && !tc::mbar_wait(&empty[s], ph ^ 1u, abort_flag, a.err)) {
                        ok = false;
                        break;
                    }
                    if (!BRANGE(((size_t)tb.x * a.nkbt + kb) * NS * blk, (size_t)NS * blk, a.lim_Xd, a.err, BC_CT_A) ||
                        !BRANGE((size_t)(tb.y / 2) * a.nkbt * NS * blk + (size_t)(tb.y % 2) * (CT_N * MK) +
                                    ((size_t)kb * NS + NS - 1) * blk,
                                CT_N * MK, a.lim_Yd, a.err, BC_CT_B)) {
                        *abort_flag = 1;
                        ok = false;
                        break;
                    }
                    uint8_t* st = smem + (size_t)s * STAGE;
                    tc::mbar_arrive_expect_tx(&full[s], (uint32_t)STAGE);
                    tc::bulk_load(st, pa + (size_t)kb * NS * blk, (uint32_t)(NS * BF_SLICE), &full[s]);
                    for (int t = 0; t < NS; ++t)
                        tc::bulk_load(st + OFF_B + t * (CT_N * MK * 2), pb + ((size_t)kb * NS + t) * blk, CT_N * MK * 2,
                                      &full[s]);
                    if (++s == a.stages) {
                        s = 0;
                        ph ^= 1u;
                    }
                }
            }
        }
    } else if (threadIdx.x == 32) {
        // ---- MMA issuer: per group one accumulation run; per k block every A slice against
        // the B slices of its levels, both operands from the stage
        int s = 0;
        uint32_t ph = 0;
        int gi = 0;
        const uint32_t smem_base = tc::smem_u32(smem);
        const uint32_t id = tc::idesc_bf16_f32(MM, CT_N, false);
        const uint64_t b_step = (uint64_t)((CT_N * MK * 2) >> 4);
        bool ok = true;
        for (int item = blockIdx.x; ok && item < a.n_items && !*abort_flag; item += gridDim.x) {
            int tile, g0, g1;
            ct_item(a, item, tile, g0, g1);
            for (int g = g0; ok && g < g1; ++g, ++gi) {
                if (gi > 0 && !tc::mbar_wait(&tempty[0], (uint32_t)((gi - 1) & 1), abort_flag, a.err)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                uint32_t d[NA];
#pragma unroll
                for (int L = 0; L < NA; ++L) d[L] = tmem + (uint32_t)(L * CT_N);
                const int kb0 = ct_kb0(a, g), kb1 = ct_kb1(a, g);
                for (int kb = kb0; ok && kb < kb1; ++kb) {
                    if (!tc::mbar_wait(&full[s], ph, abort_flag, a.err)) {
                        ok = false;
                        break;
                    }
                    const uint64_t dB = tc::sdesc_kmajor(smem_base + (uint32_t)(s * STAGE + OFF_B));
                    const bool first = kb == kb0;
#pragma unroll
                    for (int j = 0; j < NS; ++j) {
                        const uint64_t dA = tc::sdesc_kmajor(smem_base + (uint32_t)(s * STAGE + j * BF_SLICE));
                        issue_slice_gjs<NS, NA, MAXL>(j, d, dA, dB, b_step, id, first);
                    }
                    tc::mma_commit(&empty[s]);
                    if (++s == a.stages) {
                        s = 0;
                        ph ^= 1u;
                    }
                }
                tc::mma_commit(&tfull[0]);
            }
        }
    } else if (warp >= 2) {
        // ---- epilogue (warps 2-9, TMEM lane quarter warp % 4, 32 columns each): per group,
        // scale the accumulators and add them into a double-float running sum; one FP64 tile
        // per item
        const int q = warp % 4;
        const int half = warp >= 6 ? 1 : 0;
        const int r = q * 32 + (threadIdx.x % 32);
        const uint32_t lane_base = tmem + ((uint32_t)(q * 32) << 16);
        constexpr int HC = CT_N / 2;
        int gi = 0;
        bool ok = true;
        for (int item = blockIdx.x; ok && item < a.n_items; item += gridDim.x) {
            int tile, g0, g1;
            ct_item(a, item, tile, g0, g1);
            const int2 tb = a.tiles[tile];
            const int m = tb.x * MM + r;
            const int n0 = tb.y * CT_N + half * HC;
            float RH[HC], RL[HC];
#pragma unroll
            for (int c = 0; c < HC; ++c) RH[c] = RL[c] = 0.f;
            for (int g = g0; g < g1; ++g, ++gi) {
                ok = tc::mbar_wait(&tfull[0], (uint32_t)(gi & 1), abort_flag, a.err);
                __syncwarp();
                if (!ok || *abort_flag) {
                    ok = false;
                    break;
                }
                if (!BCHK((size_t)g * a.lds_x + m < a.lim_Sx, a.err, BC_CT_S, (size_t)g * a.lds_x + m, a.lim_Sx) ||
                    !BRANGE((size_t)g * a.lds_y + n0, HC, a.lim_Sy, a.err, BC_CT_S)) {
                    *abort_flag = 1;
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const float rs = a.Sx[(size_t)g * a.lds_x + m];
                const float* cs = a.Sy + (size_t)g * a.lds_y + n0;
#pragma unroll
                for (int c0 = 0; c0 < HC; c0 += 4) {
                    uint32_t v[NA][4];
#pragma unroll
                    for (int L = 0; L < NA; ++L)
                        tc::tmem_ld4_nowait(lane_base + (uint32_t)(L * CT_N + half * HC + c0), v[L]);
                    tc::tmem_wait_ld();
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        float acc[NA];
#pragma unroll
                        for (int L = 0; L < NA; ++L) acc[L] = __uint_as_float(v[L][j]);
                        float hi, lo;
                        if constexpr (NA == 6)
                            combine6(acc, hi, lo);
                        else
                            combine_n<NA>(acc, hi, lo);
                        const float sc = rs * cs[c0 + j];
                        df_add(RH[c0 + j], RL[c0 + j], hi * sc, lo * sc);
                    }
                }
                tc::tc_fence_before();
                __syncwarp();
                if ((threadIdx.x % 32) == 0) tc::mbar_arrive(&tempty[0]);
            }
            if (!ok) break;
            if constexpr (DIRECT) {
                // general product: the rows and columns that exist, (+)= into out
                const int nv = min(HC, a.N - n0);
                if (m < a.M && (nv <= 0 || BRANGE((size_t)m * a.ldo + n0, nv, a.lim_out, a.err, BC_CT_OUT))) {
                    double* dst = a.out + (size_t)m * a.ldo + n0;
#pragma unroll
                    for (int c = 0; c < HC; ++c)
                        if (c < nv) {
                            const double v = (double)RH[c] + (double)RL[c];
                            dst[c] = a.accumulate ? dst[c] + v : v;
                        }
                }
            } else {
                double* dst = a.part + (((size_t)(item / a.ntiles) * a.ntiles + tile) * MM + r) * CT_N + half * HC;
                if (!BRANGE((size_t)(dst - a.part), HC, a.lim_out, a.err, BC_CT_OUT)) continue;
#pragma unroll
                for (int c = 0; c < HC; c += 2)
                    *reinterpret_cast<double2*>(dst + c) =
                        make_double2((double)RH[c] + (double)RL[c], (double)RH[c + 1] + (double)RL[c + 1]);
            }
        }
    }
    __syncwarp();
    if (*abort_flag && threadIdx.x == 0) {
        uint64_t t0 = tc::global_timer();
        while (tc::global_timer() - t0 < 10000000ull) {
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 512u);
}

// K[m][n] (and its mirror), m >= n, = [K +] sum over splits (fixed order) of the partial tiles.
__global__ void oz_reduce_kernel(const double* __restrict__ part, int nsplit, int ntiles, int nbf,
                                 const int* __restrict__ tob, int ncb, double* __restrict__ K, int accumulate,
                                 size_t lim_part, int* __restrict__ err) {
    const size_t n_lower = (size_t)nbf * (nbf + 1) / 2;
    const size_t tstride = (size_t)ntiles * MM * CT_N;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n_lower; p += (size_t)gridDim.x * blockDim.x) {
        size_t m = (size_t)((sqrt(8.0 * (double)p + 1.0) - 1.0) * 0.5);
        while (m * (m + 1) / 2 > p) --m;
        while ((m + 1) * (m + 2) / 2 <= p) ++m;
        const size_t n = p - m * (m + 1) / 2;
        const int t = tob[(m / MM) * ncb + n / CT_N];
        const size_t off = ((size_t)t * MM + (m % MM)) * CT_N + (n % CT_N);
        if (!BCHK(t >= 0, err, BC_RED, t, ntiles) ||
            !BRANGE((size_t)(nsplit - 1) * tstride + off, 1, lim_part, err, BC_RED))
            continue;
        double s = 0.0;
        for (int k = 0; k < nsplit; ++k) s += part[(size_t)k * tstride + off];
        if (accumulate) s += K[m * nbf + n];
        K[m * nbf + n] = s;
        K[n * nbf + m] = s;
    }
}

// ---------------------------------------------------------------- general product C (+)= A B
// Digits for the contraction kernel run as a general GEMM (the metric contraction
// B = J^-1/2 (P|mn)): A (M x K, row-major) gives the row operand with one exponent per
// (row, group of RUN_K k), B (K x N, row-major) the column operand, transposed, with one
// exponent per (column, group).  Both land in [block of 128][kbt][8][128][32] pre-swizzled
// BF16 slices; rows/columns past M/N and k past K are zero digits.  Eight digits (55-bit
// fixed point) and levels up to 8, with level 5 exact as well: J^-1/2 has entries ~50x the
// largest element of B that cancel in the product, and the error of the digit form scales
// with the row and column maxima rather than with each term.

// Exponent and weight of A's row m in group g: one warp per (m, g).
__global__ void oz_gemm_rowexp_kernel(const double* __restrict__ A, size_t lda, int M, int K, int kw, int ngroups,
                                      int M_pad, int* __restrict__ Ea, float* __restrict__ Sa, int* __restrict__ err) {
    const int wid = (int)((blockIdx.x * (size_t)blockDim.x + threadIdx.x) / 32), lane = threadIdx.x % 32;
    if (wid >= M_pad * ngroups) return;
    const int m = wid % M_pad, g = wid / M_pad;
    unsigned long long mx = 0;
    if (m < M) {
        const int k1 = min(K, (g + 1) * kw);
        for (int k = g * kw + lane; k < k1; k += 32) {
            const unsigned long long b = (unsigned long long)__double_as_longlong(A[(size_t)m * lda + k]) & 0x7FFFFFFFFFFFFFFFull;
            mx = b > mx ? b : mx;
        }
    }
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) {
        const int E = exp_of_max_d(mx);
        Ea[(size_t)g * M_pad + m] = E;
        Sa[(size_t)g * M_pad + m] = scale_of(E);
        if (mx >= NONFINITE_BITS) atomicOr(err, DEV_ERR_NUMERIC);
    }
}

// Exponent and weight of B's column n in group g: one thread per (n, g), coalesced over n.
__global__ void oz_gemm_colexp_kernel(const double* __restrict__ B, size_t ldb, int N, int K, int kw, int ngroups,
                                      int N_pad, int* __restrict__ Eb, float* __restrict__ Sb, int* __restrict__ err) {
    const size_t id = blockIdx.x * (size_t)blockDim.x + threadIdx.x;
    if (id >= (size_t)N_pad * ngroups) return;
    const int n = (int)(id % N_pad), g = (int)(id / N_pad);
    unsigned long long mx = 0;
    if (n < N) {
        const int k1 = min(K, (g + 1) * kw);
        for (int k = g * kw; k < k1; ++k) {
            const unsigned long long b = (unsigned long long)__double_as_longlong(B[(size_t)k * ldb + n]) & 0x7FFFFFFFFFFFFFFFull;
            mx = b > mx ? b : mx;
        }
    }
    const int E = exp_of_max_d(mx);
    Eb[(size_t)g * N_pad + n] = E;
    Sb[(size_t)g * N_pad + n] = scale_of(E);
    if (mx >= NONFINITE_BITS) atomicOr(err, DEV_ERR_NUMERIC);
}

// Eight consecutive values -> the GM_NS BF16 slices of their digits, packed in uint4s.
__device__ __forceinline__ void digits8(const double* x, int E, uint32_t (&w)[GM_NS][4]) {
    const unsigned long long off = digit_off<GM_NS>();
#pragma unroll
    for (int j = 0; j < 8; ++j) {
        const unsigned long long uu = (unsigned long long)(fix_dn<GM_NS>(x[j], E) + (long long)off);
#pragma unroll
        for (int s = 0; s < GM_NS; ++s) {
            const uint32_t bits = field_bf16(digit_field_n<GM_NS>(uu, s), slice_weight(s));
            if (j % 2 == 0)
                w[s][j / 2] = bits;
            else
                w[s][j / 2] |= bits << 16;
        }
    }
}
__device__ __forceinline__ void store_slices(__nv_bfloat16* base, int r, int c, const uint32_t (&w)[GM_NS][4]) {
    const uint32_t off = tc::swz_offset((uint32_t)r, (uint32_t)c) / 2;
#pragma unroll
    for (int s = 0; s < GM_NS; ++s)
        *reinterpret_cast<uint4*>(base + (size_t)s * (MM * MK) + off) = make_uint4(w[s][0], w[s][1], w[s][2], w[s][3]);
}

// Row operand: unit = (row, 8 consecutive k); units ordered (block, kb, row, chunk) so that a
// warp reads 8 rows x 256 contiguous bytes.
__global__ void __launch_bounds__(256) oz_gemm_split_A_kernel(const double* __restrict__ A, size_t lda, int M, int K,
                                                              int M_pad, int nkbt, int kpg, const int* __restrict__ Ea,
                                                              __nv_bfloat16* __restrict__ Xd) {
    const size_t total = (size_t)M_pad * nkbt * (MK / 8);
    for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < total; u += (size_t)gridDim.x * blockDim.x) {
        const int c = (int)(u % (MK / 8));
        const int r = (int)((u / (MK / 8)) % MM);
        const size_t bk = u / (MM * (MK / 8));  // mb * nkbt + kb
        const int kb = (int)(bk % nkbt), mb = (int)(bk / nkbt);
        const int m = mb * MM + r, k0 = kb * MK + c * 8;
        const int E = Ea[(size_t)(kb / kpg) * M_pad + m];
        double x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = (m < M && k0 + j < K) ? A[(size_t)m * lda + k0 + j] : 0.0;
        uint32_t w[GM_NS][4];
        digits8(x, E, w);
        store_slices(Xd + bk * GM_NS * (MM * MK), r, c, w);
    }
}

// Column operand (B transposed): unit = (column n, 8 consecutive k); consecutive threads take
// consecutive columns, so each of the eight row reads is coalesced.
__global__ void __launch_bounds__(256) oz_gemm_split_Bt_kernel(const double* __restrict__ B, size_t ldb, int N, int K,
                                                               int N_pad, int nkbt, int kpg, const int* __restrict__ Eb,
                                                               __nv_bfloat16* __restrict__ Yd) {
    const size_t total = (size_t)N_pad * nkbt * (MK / 8);
    for (size_t u = blockIdx.x * (size_t)blockDim.x + threadIdx.x; u < total; u += (size_t)gridDim.x * blockDim.x) {
        const int n = (int)(u % N_pad);
        const size_t kc = u / N_pad;  // kb * 4 + chunk
        const int kb = (int)(kc / (MK / 8)), c = (int)(kc % (MK / 8));
        const int k0 = kb * MK + c * 8;
        const int E = Eb[(size_t)(kb / kpg) * N_pad + n];
        double x[8];
#pragma unroll
        for (int j = 0; j < 8; ++j) x[j] = (n < N && k0 + j < K) ? B[(size_t)(k0 + j) * ldb + n] : 0.0;
        uint32_t w[GM_NS][4];
        digits8(x, E, w);
        store_slices(Yd + ((size_t)(n / MM) * nkbt + kb) * GM_NS * (MM * MK), n % MM, c, w);
    }
}

}  // namespace oz

// ---------------------------------------------------------------- host side
struct OzState {
    int nbf_p = 0;
    uint8_t* Bd = nullptr;                 // int8 digit fields of B
    float* sA = nullptr;                   // row weights of B
    unsigned long long* rowmax = nullptr;  // row maxima of |B| (bits)
    bool B_ready = false;
    int* eC = nullptr;
    float* sC = nullptr;
    __nv_bfloat16* Cd = nullptr;
    size_t C_cap = 0, sc_cap = 0;
    float2* Xdf = nullptr;
    __nv_bfloat16* Xd = nullptr;
    size_t X_cap = 0;  // (aux function, occupied column) pairs the X buffers hold: qb * nocc_p
    unsigned* xmax = nullptr;
    float* Sx = nullptr;
    size_t xm_cap = 0, sx_cap = 0;
    double* part = nullptr;
    size_t part_cap = 0;
    int2* d_tiles = nullptr;
    int* d_tob = nullptr;
    int tiles_nbf_p = 0, ntiles = 0, ncb = 0;
    int* err = nullptr;
    int num_sms = 0;
    bool attrs_set = false;
    std::vector<cudaEvent_t> tr_ev;  // begin/end of each batch's half-transform, last build
    int n_tr = 0;
    // (128-row block, 32-wide k block) pairs of B that touch a stored tile, grouped by row block
    int* d_mb_ptr = nullptr;
    int* d_mb_kb = nullptr;
    int* d_blk_mb = nullptr;
    int nnz = 0, lists_nbf_p = 0;
    // non-symmetric builds (C_left != C_right): digits of C_right and of its X, all tiles
    int* eC_r = nullptr;
    float* sC_r = nullptr;
    __nv_bfloat16* Cd_r = nullptr;
    size_t Cr_cap = 0, scr_cap = 0;
    __nv_bfloat16* Xd_r = nullptr;
    size_t Xr_cap = 0;  // the same for the right factor's digits
    float* Sx_r = nullptr;
    size_t sxr_cap = 0;
    int2* d_tiles_all = nullptr;
    int tiles_all_nbf_p = 0, ntiles_all = 0;
};

OzState* oz_create() { return new OzState(); }

float oz_last_transform_ms(OzState* o) {
    if (!o) return 0.f;
    float total = 0.f;
    for (int b = 0; b < o->n_tr; ++b) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, o->tr_ev[2 * b], o->tr_ev[2 * b + 1]) == cudaSuccess) total += ms;
    }
    return total;
}

namespace {

int oz_alloc(void** p, size_t bytes, std::string& err) {
    if (*p) {
        cudaFree(*p);
        *p = nullptr;
    }
    cudaError_t e = engine_malloc(p, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        err = "emulated FP64: device allocation of " + std::to_string(bytes / 1e9) + " GB refused";
        return GDFJK_ERR_OOM;
    }
    return GDFJK_OK;
}

void oz_free(void** p) {
    big_free(*p);
    *p = nullptr;
}


double x_cap_bytes() {
    const char* s = getenv("GDFJK_OZ_XCAP_GB");
    double gb = s ? atof(s) : 24.0;
    if (!(gb > 0.0)) gb = 24.0;
    return gb * 1e9;
}

}  // namespace

void oz_release(OzState* o) {
    if (!o) return;
    oz_free((void**)&o->Bd);
    oz_free((void**)&o->sA);
    oz_free((void**)&o->rowmax);
    oz_free((void**)&o->Xdf);
    oz_free((void**)&o->Xd);
    oz_free((void**)&o->Xd_r);
    o->X_cap = 0;
    o->Xr_cap = 0;
    o->B_ready = false;
}

void oz_invalidate(OzState* o) {
    if (!o) return;
    oz_free((void**)&o->Bd);
    o->B_ready = false;
}

void oz_destroy(OzState* o) {
    if (!o) return;
    oz_release(o);
    void* ps[] = {o->eC, o->sC, o->Cd, o->xmax, o->Sx, o->part, o->d_tiles, o->d_tob, o->err, o->d_mb_ptr, o->d_mb_kb,
                  o->d_blk_mb, o->eC_r, o->sC_r, o->Cd_r, o->Sx_r, o->d_tiles_all};
    for (void* p : ps)
        if (p) cudaFree(p);
    for (cudaEvent_t e : o->tr_ev) cudaEventDestroy(e);
    delete o;
}

size_t oz_query_memory(int nbf, int naux, int max_nocc) {
    const size_t nbf_p = (size_t)round_up(nbf, oz::MM);
    size_t b = (size_t)naux * nbf_p * nbf_p * oz::NSL;  // int8 digits of B
    b += (size_t)naux * nbf_p * 12;                     // row maxima and weights
    const size_t nocc_p = (size_t)round_up(std::max(1, max_nocc), 32);
    const size_t per_q = nocc_p * ((size_t)nbf * 8 + nbf_p * oz::NSL * 2);
    b += std::min((size_t)naux * per_q, (size_t)x_cap_bytes() + per_q * 2048);
    return b;
}

int oz_error_flag(OzState* o, cudaStream_t s) {
    if (!o || !o->err) return 0;
    int f = 0;
    cudaMemcpyAsync(&f, o->err, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (f) cudaMemsetAsync(o->err, 0, sizeof(int), s);
    return f;
}

namespace {

using CtKernel = void (*)(const oz::CtArgs);
// The contraction's instantiations: K = X X^T (partial tiles), the general product (8 digits,
// direct), the non-symmetric K (direct).
CtKernel ct_sym_kernel() { return oz::oz_contract_kernel<oz::NSL, oz::CT_NACC, oz::NSL - 1, false>; }
CtKernel ct_gemm_kernel() { return oz::oz_contract_kernel<oz::GM_NS, oz::GM_NACC, oz::GM_MAXL, true>; }
CtKernel ct_nonsym_kernel() { return oz::oz_contract_kernel<oz::NSL, oz::CT_NACC, oz::NSL - 1, true>; }

// error word, SM count and kernel attributes, once per state
int oz_prepare(OzState* o, cudaStream_t s, std::string& err) {
    using namespace oz;
    int rc;
    if (!o->err) {
        if ((rc = oz_alloc((void**)&o->err, sizeof(int), err))) return rc;
        cudaMemsetAsync(o->err, 0, sizeof(int), s);
    }
    if (!o->num_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&o->num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (o->num_sms <= 0) o->num_sms = 152;
    }
    if (!o->attrs_set) {
        cudaFuncSetAttribute(oz_transform_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BUDGET);
        cudaFuncSetAttribute(ct_sym_kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BUDGET);
        cudaFuncSetAttribute(ct_gemm_kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BUDGET);
        cudaFuncSetAttribute(ct_nonsym_kernel(), cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BUDGET);
        o->attrs_set = true;
    }
    return GDFJK_OK;
}

}  // namespace

// The digit copy of B on `o` (once per upload): the (row block, k block) pairs of B that touch
// a stored tile, then the int8 digit fields of those blocks.
static int oz_ensure_digits(OzState* o, const double* B, const TileLayout& L, const int* map_host, int nbf, int naux,
                            cudaStream_t s, std::string& err) {
    using namespace oz;
    int rc;
    const int nbf_p = round_up(nbf, MM);
    if ((rc = oz_prepare(o, s, err))) return rc;
    // ---- the (row block, k block) pairs of B that touch a stored tile (the tile map is fixed)
    if (o->lists_nbf_p != nbf_p) {
        const BlockLists bl = build_block_lists(map_host, L.nT, nbf_p, MM, MK, TILE);
        const std::vector<int>& ptr = bl.ptr;
        const std::vector<int>& kbs = bl.kb;
        const std::vector<int>& bmb = bl.mb;
        if (kbs.empty()) {
            err = "emulated FP64: B has no stored tiles";
            return GDFJK_ERR_ARG;
        }
        if ((rc = oz_alloc((void**)&o->d_mb_ptr, ptr.size() * sizeof(int), err)) ||
            (rc = oz_alloc((void**)&o->d_mb_kb, kbs.size() * sizeof(int), err)) ||
            (rc = oz_alloc((void**)&o->d_blk_mb, bmb.size() * sizeof(int), err)))
            return rc;
        cudaMemcpy(o->d_mb_ptr, ptr.data(), ptr.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(o->d_mb_kb, kbs.data(), kbs.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(o->d_blk_mb, bmb.data(), bmb.size() * sizeof(int), cudaMemcpyHostToDevice);
        o->nnz = (int)kbs.size();
        o->lists_nbf_p = nbf_p;
        o->B_ready = false;
    }
    // ---- digits of B (once per upload), the listed blocks only
    if (!o->B_ready || o->nbf_p != nbf_p) {
        const size_t rows = (size_t)naux * nbf_p;
        o->B_ready = false;
        if ((rc = oz_alloc((void**)&o->rowmax, rows * 8, err)) || (rc = oz_alloc((void**)&o->sA, rows * 4, err)) ||
            (rc = oz_alloc((void**)&o->Bd, (size_t)naux * o->nnz * I8_BLOCK, err)))
            return rc;
        cudaMemsetAsync(o->rowmax, 0, rows * 8, s);
        if (L.ntiles > 0)
            oz_rowmax_kernel<<<(unsigned)((size_t)naux * L.ntiles), 256, 0, s>>>(B, L.ntiles, L.tI, L.tJ, nbf_p, o->rowmax,
                                                                                   o->err);
        oz_split_B_kernel<<<(unsigned)((size_t)naux * o->nnz), 256, 0, s>>>(
            B, nbf, L.nT, L.ntiles, L.map, nbf_p, o->nnz, o->d_blk_mb, o->d_mb_kb, o->d_mb_ptr, o->rowmax, o->sA, o->Bd);
        o->nbf_p = nbf_p;
        o->B_ready = true;
    }
    return GDFJK_OK;
}

int oz_build_K(OzState* o, const double* B, const TileLayout& L, const int* map_host, int nbf, int naux, const double* Cpad,
               const double* Crpad, int nocc, int nocc_pad, double* K, cudaEvent_t ev_transform_done, cudaStream_t s,
               std::string& err, OzState* o_right, const double* B_right, const TileLayout* L_right) {
    using namespace oz;
    int rc;
    const int nbf_p = round_up(nbf, MM);
    const int nmb = nbf_p / MM, nkb = nbf_p / MK;
    if ((rc = oz_ensure_digits(o, B, L, map_host, nbf, naux, s, err))) return rc;
    if (o_right) {  // K from two tensors: C_right's half-transform reads the other digit copy
        if ((rc = oz_ensure_digits(o_right, B_right, *L_right, map_host, nbf, naux, s, err))) return rc;
        if (!Crpad) Crpad = Cpad;
    }
    if (nocc_pad > RUN_K) {
        // one aux function's columns must fit one exact contraction run (levels 0-3 provably exact)
        err = "emulated FP64: nocc above " + std::to_string(RUN_K) + " is not supported (use the native FP64 K)";
        return GDFJK_ERR_ARG;
    }
    // ---- digits of C^T, in column chunks of <= 80 (five accumulators of N columns and seven
    // 16-column A slots fill the 512 TMEM columns at N = 80; three pipeline stages in shared
    // memory)
    const int nocc_p = nocc_pad;
    const int nchunk = (nocc_p + TR_MAX_N - 1) / TR_MAX_N;
    const int N = round_up((nocc_p + nchunk - 1) / nchunk, 16);
    const int ncols = nchunk * N;
    if ((size_t)ncols > o->sc_cap) {
        o->sc_cap = 0;
        if ((rc = oz_alloc((void**)&o->eC, ncols * sizeof(int), err)) || (rc = oz_alloc((void**)&o->sC, ncols * 4, err)))
            return rc;
        o->sc_cap = ncols;
    }
    const size_t ce = (size_t)ncols * nbf_p * NSL;
    if (ce > o->C_cap) {
        o->C_cap = 0;
        if ((rc = oz_alloc((void**)&o->Cd, ce * 2, err))) return rc;
        o->C_cap = ce;
    }
    const bool nonsym = Crpad != nullptr;
    if (nonsym) {
        if ((size_t)ncols > o->scr_cap) {
            o->scr_cap = 0;
            if ((rc = oz_alloc((void**)&o->eC_r, ncols * sizeof(int), err)) ||
                (rc = oz_alloc((void**)&o->sC_r, ncols * 4, err)))
                return rc;
            o->scr_cap = ncols;
        }
        if (ce > o->Cr_cap) {
            o->Cr_cap = 0;
            if ((rc = oz_alloc((void**)&o->Cd_r, ce * 2, err))) return rc;
            o->Cr_cap = ce;
        }
    }
    for (int side = 0; side < (nonsym ? 2 : 1); ++side) {
        const double* Cs = side ? Crpad : Cpad;
        int* eCs = side ? o->eC_r : o->eC;
        float* sCs = side ? o->sC_r : o->sC;
        __nv_bfloat16* Cds = side ? o->Cd_r : o->Cd;
        oz_col_scale_kernel<<<ncols, 256, 0, s>>>(Cs, nbf, nocc_pad, nocc, eCs, sCs, o->err);
        const size_t total = (size_t)ncols * (nbf_p / 8);
        const int blocks = (int)std::min<size_t>((total + 255) / 256, (size_t)o->num_sms * 8);
        oz_split_C_kernel<<<blocks, 256, 0, s>>>(Cs, nbf, nbf_p, nocc_pad, N, ncols, eCs, Cds);
    }
    // ---- batches of aux functions (multiples of the group size) bounded by the X buffers
    const int G = std::max(1, RUN_K / nocc_p);
    const double per_q = (double)nocc_p * ((double)nbf * 8.0 + (nonsym ? 2.0 : 1.0) * (double)nbf_p * NSL * 2.0);
    int qb = (int)std::min<double>((double)naux, std::max<double>(G, std::floor(x_cap_bytes() / per_q / G) * G));
    qb = std::max(1, qb);
    // capacity in (aux function, column) pairs, not in aux functions: a later build with more
    // occupied columns gets a smaller batch whose buffers may still need to be larger
    const size_t x_need = (size_t)qb * nocc_p;
    if (x_need > o->X_cap) {
        o->X_cap = 0;
        if ((rc = oz_alloc((void**)&o->Xdf, (size_t)nbf * x_need * 8, err)) ||
            (rc = oz_alloc((void**)&o->Xd, (size_t)nbf_p * x_need * NSL * 2, err)))
            return rc;
        o->X_cap = x_need;
    }
    const int ngroups_max = (qb + G - 1) / G;
    if ((size_t)nbf * ngroups_max > o->xm_cap) {
        o->xm_cap = 0;
        if ((rc = oz_alloc((void**)&o->xmax, (size_t)nbf * ngroups_max * 4, err))) return rc;
        o->xm_cap = (size_t)nbf * ngroups_max;
    }
    if ((size_t)nbf_p * ngroups_max > o->sx_cap) {
        o->sx_cap = 0;
        if ((rc = oz_alloc((void**)&o->Sx, (size_t)nbf_p * ngroups_max * 4, err))) return rc;
        o->sx_cap = (size_t)nbf_p * ngroups_max;
    }
    if (nonsym) {
        if (x_need > o->Xr_cap) {
            o->Xr_cap = 0;
            if ((rc = oz_alloc((void**)&o->Xd_r, (size_t)nbf_p * x_need * NSL * 2, err))) return rc;
            o->Xr_cap = x_need;
        }
        if ((size_t)nbf_p * ngroups_max > o->sxr_cap) {
            o->sxr_cap = 0;
            if ((rc = oz_alloc((void**)&o->Sx_r, (size_t)nbf_p * ngroups_max * 4, err))) return rc;
            o->sxr_cap = (size_t)nbf_p * ngroups_max;
        }
        // every (128-row block, 64-column block) of K, row-block-major
        if (o->tiles_all_nbf_p != nbf_p) {
            std::vector<int2> tl;
            for (int I = 0; I < nmb; ++I)
                for (int Jc = 0; Jc < nbf_p / CT_N; ++Jc) tl.push_back(make_int2(I, Jc));
            if ((rc = oz_alloc((void**)&o->d_tiles_all, tl.size() * sizeof(int2), err))) return rc;
            cudaMemcpy(o->d_tiles_all, tl.data(), tl.size() * sizeof(int2), cudaMemcpyHostToDevice);
            o->ntiles_all = (int)tl.size();
            o->tiles_all_nbf_p = nbf_p;
        }
    }
    // ---- contraction tiles: (128-row block, 64-row block) pairs of the lower triangle
    if (o->tiles_nbf_p != nbf_p) {
        const int ncb = nbf_p / CT_N;
        std::vector<int2> tl;
        std::vector<int> tob((size_t)nmb * ncb, -1);
        for (int I = 0; I < nmb; ++I)
            for (int Jc = 0; Jc < ncb && Jc * CT_N < (I + 1) * MM; ++Jc) {
                tob[(size_t)I * ncb + Jc] = (int)tl.size();
                tl.push_back(make_int2(I, Jc));
            }
        if ((rc = oz_alloc((void**)&o->d_tiles, tl.size() * sizeof(int2), err)) ||
            (rc = oz_alloc((void**)&o->d_tob, tob.size() * sizeof(int), err)))
            return rc;
        cudaMemcpy(o->d_tiles, tl.data(), tl.size() * sizeof(int2), cudaMemcpyHostToDevice);
        cudaMemcpy(o->d_tob, tob.data(), tob.size() * sizeof(int), cudaMemcpyHostToDevice);
        o->ntiles = (int)tl.size();
        o->ncb = ncb;
        o->tiles_nbf_p = nbf_p;
    }
    const int tr_stage = TR_OFF_C + NSL * N * MK * 2;
    const int tr_stages = std::min(4, (SMEM_BUDGET - SMEM_RESERVE - 4 * ncols) / tr_stage);
    const int ct_stages = std::min(4, (SMEM_BUDGET - SMEM_RESERVE) / CT_STAGE);
    if (tr_stages < 2 || ct_stages < 2) {
        err = "emulated FP64: pipeline stages do not fit in shared memory";
        return GDFJK_ERR_ARG;
    }
    const int nbatch = (naux + qb - 1) / qb;
    const int nsides = nonsym ? 2 : 1;  // half-transforms per batch, each timed by an event pair
    while ((int)o->tr_ev.size() < 2 * nsides * nbatch) {
        cudaEvent_t e;
        if (cudaEventCreate(&e) != cudaSuccess) {
            err = "emulated FP64: cudaEventCreate failed";
            return GDFJK_ERR_CUDA;
        }
        o->tr_ev.push_back(e);
    }
    o->n_tr = nsides * nbatch;
    for (int q0 = 0, batch = 0; q0 < naux; q0 += qb, ++batch) {
        const int nq = std::min(qb, naux - q0);
        const int ngroups = (nq + G - 1) / G;
        const size_t kdim_b = (size_t)nq * nocc_p;
        const size_t nkbt = kdim_b / MK;
        for (int side = 0; side < nsides; ++side) {
            // X = B C (side 0: C_left, 1: C_right) -> its digits and group weights
            cudaMemsetAsync(o->xmax, 0, (size_t)nbf * ngroups * 4, s);
            const OzState* ob = (side && o_right) ? o_right : o;  // digits of the tensor this side reads
            TrArgs ta{};
            ta.Bd = ob->Bd;
            ta.Cd = side ? o->Cd_r : o->Cd;
            ta.sA = ob->sA;
            ta.sC = side ? o->sC_r : o->sC;
            ta.Xdf = o->Xdf;
            ta.xmax = o->xmax;
            ta.q0 = q0;
            ta.nq = nq;
            ta.nmb = nmb;
            ta.nkb = nkb;
            ta.nbf = nbf;
            ta.nbf_p = nbf_p;
            ta.nocc_p = nocc_p;
            ta.N = N;
            ta.nchunk = nchunk;
            ta.G = G;
            ta.ngroups = ngroups;
            ta.kdim_b = kdim_b;
            ta.stages = tr_stages;
            ta.mb_ptr = ob->d_mb_ptr;
            ta.mb_kb = ob->d_mb_kb;
            ta.nnz = ob->nnz;
            ta.ncols = ncols;
            ta.run_kb = TR_RUN_K / MK;
            ta.nbuf = (2 * TR_NACC * N <= TR_ACOL0) ? 2 : 1;
            ta.n_items = nq * nmb * nchunk;
            ta.err = o->err;
            ta.lim_Bd = (size_t)naux * ob->nnz * I8_BLOCK;
            ta.lim_Cd = side ? o->Cr_cap : o->C_cap;
            ta.lim_X = (size_t)nbf * o->X_cap;
            ta.lim_xmax = o->xm_cap;
            ta.lim_sA = (size_t)naux * nbf_p;
            const int ev = 2 * (nsides * batch + side);
            cudaEventRecord(o->tr_ev[ev], s);
            oz_transform_kernel<<<(unsigned)std::min(ta.n_items, o->num_sms), TR_THREADS, SMEM_BUDGET, s>>>(ta);
            cudaEventRecord(o->tr_ev[ev + 1], s);
            // the transform phase ends with the last batch's last half-transform kernel
            if (ev_transform_done && q0 + qb >= naux && side == nsides - 1) cudaEventRecord(ev_transform_done, s);
            oz_split_X_kernel<<<dim3((unsigned)nmb, (unsigned)ngroups), 256, 0, s>>>(
                o->Xdf, o->xmax, nbf, nbf_p, ngroups, G, nq, nocc_p, kdim_b, nkbt, side ? o->Sx_r : o->Sx,
                side ? o->Xd_r : o->Xd, (size_t)nbf * o->X_cap, (size_t)nbf_p * (side ? o->Xr_cap : o->X_cap) * NSL,
                side ? o->sxr_cap : o->sx_cap, o->err);
        }
        if (nonsym) {
            // K (+)= X_left X_right^T over every tile, written straight into K (nbf x nbf)
            CtArgs ca{};
            ca.Xd = o->Xd;
            ca.Yd = o->Xd_r;
            ca.Sx = o->Sx;
            ca.Sy = o->Sx_r;
            ca.tiles = o->d_tiles_all;
            ca.ntiles = o->ntiles_all;
            ca.nsplit = 1;
            ca.gps = ngroups;
            ca.ngroups = ngroups;
            ca.kpg = G * nocc_p / MK;
            ca.nkb = (int)nkbt;
            ca.lds_x = ca.lds_y = nbf_p;
            ca.nkbt = nkbt;
            ca.part = nullptr;
            ca.out = K;
            ca.ldo = (size_t)nbf;
            ca.M = ca.N = nbf;
            ca.accumulate = batch > 0 ? 1 : 0;
            ca.stages = ct_stages;
            ca.n_items = o->ntiles_all;
            ca.err = o->err;
            ca.lim_Xd = (size_t)nbf_p * o->X_cap * NSL;
            ca.lim_Yd = (size_t)nbf_p * o->Xr_cap * NSL;
            ca.lim_Sx = o->sx_cap;
            ca.lim_Sy = o->sxr_cap;
            ca.lim_out = (size_t)nbf * nbf;
            ct_nonsym_kernel()<<<(unsigned)std::min(ca.n_items, o->num_sms), CT_THREADS, SMEM_BUDGET, s>>>(ca);
            continue;
        }
        // split over groups so that there are about two work items per SM
        int nsplit = std::max(1, std::min(ngroups, (2 * o->num_sms + o->ntiles - 1) / o->ntiles));
        const int gps = (ngroups + nsplit - 1) / nsplit;
        nsplit = (ngroups + gps - 1) / gps;
        const size_t pe = (size_t)nsplit * o->ntiles * MM * CT_N;
        if (pe > o->part_cap) {
            o->part_cap = 0;
            if ((rc = oz_alloc((void**)&o->part, pe * 8, err))) return rc;
            o->part_cap = pe;
        }
        CtArgs ca{};
        ca.Xd = o->Xd;
        ca.Yd = o->Xd;
        ca.Sx = o->Sx;
        ca.Sy = o->Sx;
        ca.tiles = o->d_tiles;
        ca.ntiles = o->ntiles;
        ca.nsplit = nsplit;
        ca.gps = gps;
        ca.ngroups = ngroups;
        ca.kpg = G * nocc_p / MK;
        ca.nkb = (int)nkbt;
        ca.lds_x = ca.lds_y = nbf_p;
        ca.nkbt = nkbt;
        ca.part = o->part;
        ca.stages = ct_stages;
        ca.n_items = o->ntiles * nsplit;
        ca.err = o->err;
        ca.lim_Xd = ca.lim_Yd = (size_t)nbf_p * o->X_cap * NSL;
        ca.lim_Sx = ca.lim_Sy = o->sx_cap;
        ca.lim_out = o->part_cap;
        ct_sym_kernel()<<<(unsigned)std::min(ca.n_items, o->num_sms), CT_THREADS, SMEM_BUDGET, s>>>(ca);
        const size_t nl = (size_t)nbf * (nbf + 1) / 2;
        const int blocks = (int)std::min<size_t>((nl + 255) / 256, (size_t)o->num_sms * 16);
        oz_reduce_kernel<<<blocks, 256, 0, s>>>(o->part, nsplit, o->ntiles, nbf, o->d_tob, o->ncb, K, batch > 0 ? 1 : 0,
                                                 o->part_cap, o->err);
    }
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("emulated FP64: launch failed: ") + cudaGetErrorString(e);
        return GDFJK_ERR_CUDA;
    }
    return GDFJK_OK;
}

namespace {

double gemm_chunk_bytes() {
    const char* s = getenv("GDFJK_OZ_GEMM_CHUNK_GB");
    double gb = s ? atof(s) : 8.0;
    if (!(gb > 0.0)) gb = 8.0;
    return gb * 1e9;
}

// Work items of one column chunk: every (128-row block, 64-column block) pair, in strips of 16
// column blocks, row-block-major inside a strip, so that the CTAs working at the same time
// share a few row blocks of A and 16 column blocks of B in L2.
std::vector<int2> gemm_tiles(int nmb, int ncb) {
    constexpr int W = 16;
    std::vector<int2> tl;
    tl.reserve((size_t)nmb * ncb);
    for (int c0 = 0; c0 < ncb; c0 += W)
        for (int mb = 0; mb < nmb; ++mb)
            for (int c = c0; c < std::min(ncb, c0 + W); ++c) tl.push_back(make_int2(mb, c));
    return tl;
}

// device buffers of one product, released when the call returns
struct GemmBuffers {
    void* p[8] = {};
    ~GemmBuffers() {
        for (void* q : p)
            if (q) cudaFree(q);
    }
};

}  // namespace

int oz_gemm(OzState* o, const double* A, size_t lda, const double* B, size_t ldb, double* C, size_t ldc, int M, int N,
            int K, int accumulate, cudaStream_t s, std::string& err, int transb) {
    using namespace oz;
    int rc;
    if (M < 0 || N < 0 || K < 1 || !A || !B || !C || lda < (size_t)K || ldb < (size_t)(transb ? K : N) ||
        ldc < (size_t)N) {
        err = "emulated FP64 product: invalid sizes or pointers";
        return GDFJK_ERR_ARG;
    }
    if (M == 0 || N == 0) return GDFJK_OK;
    if ((rc = oz_prepare(o, s, err))) return rc;
    const int M_pad = round_up(M, MM), K_pad = round_up(K, MK);
    const int nkbt = K_pad / MK, kpg = RUN_K / MK;
    const int ngroups = (nkbt + kpg - 1) / kpg;
    const int nmb = M_pad / MM;
    // columns per chunk: digits of B (K_pad x 7 BF16 slices) within the chunk budget
    const double per_col = (double)K_pad * GM_NS * 2.0 + ngroups * 8.0 + (double)nmb * 8.0 / CT_N;
    long nc = (long)std::floor(gemm_chunk_bytes() / per_col / MM) * MM;
    nc = std::max<long>(MM, std::min<long>(nc, round_up(N, MM)));
    GemmBuffers bufs;
    __nv_bfloat16 *Xd = nullptr, *Yd = nullptr;
    int *Ea = nullptr, *Eb = nullptr;
    float *Sa = nullptr, *Sb = nullptr;
    int2* tiles = nullptr;
    if ((rc = oz_alloc(&bufs.p[0], (size_t)M_pad * K_pad * GM_NS * 2, err)) ||
        (rc = oz_alloc(&bufs.p[1], (size_t)ngroups * M_pad * 4, err)) ||
        (rc = oz_alloc(&bufs.p[2], (size_t)ngroups * M_pad * 4, err)) ||
        (rc = oz_alloc(&bufs.p[3], (size_t)nc * K_pad * GM_NS * 2, err)) ||
        (rc = oz_alloc(&bufs.p[4], (size_t)ngroups * nc * 4, err)) ||
        (rc = oz_alloc(&bufs.p[5], (size_t)ngroups * nc * 4, err)) ||
        (rc = oz_alloc(&bufs.p[6], (size_t)nmb * (nc / CT_N) * sizeof(int2), err)))
        return rc;
    Xd = (__nv_bfloat16*)bufs.p[0];
    Ea = (int*)bufs.p[1];
    Sa = (float*)bufs.p[2];
    Yd = (__nv_bfloat16*)bufs.p[3];
    Eb = (int*)bufs.p[4];
    Sb = (float*)bufs.p[5];
    tiles = (int2*)bufs.p[6];
    const int ct_stages = std::min(4, (SMEM_BUDGET - SMEM_RESERVE) / ct_stage_bytes(GM_NS));
    {
        const size_t warps = (size_t)M_pad * ngroups;
        oz_gemm_rowexp_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(A, lda, M, K, RUN_K, ngroups, M_pad, Ea,
                                                                                      Sa, o->err);
        const size_t units = (size_t)M_pad * nkbt * (MK / 8);
        const int blocks = (int)std::min<size_t>((units + 255) / 256, (size_t)o->num_sms * 16);
        oz_gemm_split_A_kernel<<<blocks, 256, 0, s>>>(A, lda, M, K, M_pad, nkbt, kpg, Ea, Xd);
    }
    int tiles_ncb = -1;
    for (long c0 = 0; c0 < N; c0 += nc) {
        const int ncc = (int)std::min<long>(nc, N - c0);
        const int N_pad = round_up(ncc, MM);
        const int ncb = N_pad / CT_N;
        if (ncb != tiles_ncb) {
            const std::vector<int2> tl = gemm_tiles(nmb, ncb);
            cudaStreamSynchronize(s);  // the previous chunk's contraction may still read the list
            cudaMemcpy(tiles, tl.data(), tl.size() * sizeof(int2), cudaMemcpyHostToDevice);
            tiles_ncb = ncb;
        }
        const size_t units = (size_t)N_pad * nkbt * (MK / 8);
        const int blocks = (int)std::min<size_t>((units + 255) / 256, (size_t)o->num_sms * 16);
        if (transb) {
            // B is N x K with K contiguous: its rows are split exactly as A's
            const double* Bc = B + (size_t)c0 * ldb;
            const size_t warps = (size_t)N_pad * ngroups;
            oz_gemm_rowexp_kernel<<<(unsigned)((warps * 32 + 255) / 256), 256, 0, s>>>(Bc, ldb, ncc, K, RUN_K, ngroups,
                                                                                          N_pad, Eb, Sb, o->err);
            oz_gemm_split_A_kernel<<<blocks, 256, 0, s>>>(Bc, ldb, ncc, K, N_pad, nkbt, kpg, Eb, Yd);
        } else {
            const size_t cols = (size_t)N_pad * ngroups;
            oz_gemm_colexp_kernel<<<(unsigned)((cols + 255) / 256), 256, 0, s>>>(B + c0, ldb, ncc, K, RUN_K, ngroups,
                                                                                  N_pad, Eb, Sb, o->err);
            oz_gemm_split_Bt_kernel<<<blocks, 256, 0, s>>>(B + c0, ldb, ncc, K, N_pad, nkbt, kpg, Eb, Yd);
        }
        CtArgs ca{};
        ca.Xd = Xd;
        ca.Yd = Yd;
        ca.Sx = Sa;
        ca.Sy = Sb;
        ca.tiles = tiles;
        ca.ntiles = nmb * ncb;
        ca.nsplit = 1;
        ca.gps = ngroups;
        ca.ngroups = ngroups;
        ca.kpg = kpg;
        ca.nkb = nkbt;
        ca.lds_x = M_pad;
        ca.lds_y = N_pad;
        ca.nkbt = (size_t)nkbt;
        ca.part = nullptr;
        ca.out = C + c0;
        ca.ldo = ldc;
        ca.M = M;
        ca.N = ncc;
        ca.accumulate = accumulate ? 1 : 0;
        ca.stages = ct_stages;
        ca.n_items = ca.ntiles;
        ca.err = o->err;
        ca.lim_Xd = (size_t)M_pad * K_pad * GM_NS;
        ca.lim_Yd = (size_t)nc * K_pad * GM_NS;
        ca.lim_Sx = (size_t)ngroups * M_pad;
        ca.lim_Sy = (size_t)ngroups * nc;
        ca.lim_out = (size_t)(M - 1) * ldc + (size_t)(N - c0);
        ct_gemm_kernel()<<<(unsigned)std::min(ca.n_items, o->num_sms), CT_THREADS, SMEM_BUDGET, s>>>(ca);
    }
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);  // the buffers are released on return
    if (e != cudaSuccess) {
        err = std::string("emulated FP64 product: ") + cudaGetErrorString(e);
        return GDFJK_ERR_CUDA;
    }
    return GDFJK_OK;
}

}  // namespace gdfjk
