// k_mixed.cu — split-precision exchange (the precision form) on the 5th-generation tensor cores.
//
// K = sum_Q B_Q U S U^T B_Q for a signed factor U S U^T of the density (S = +1 on the first
// npos columns, -1 on the rest; a full build is U = C_occ, all positive; an incremental
// build factors dD = D_new - D_old).  Two tcgen05 GEMMs with BF16 operands split in two
// (x = x_hi + x_lo, each BF16) and FP32 accumulation in tensor memory, three products per
// step (hi*hi + hi*lo + lo*hi, the "BF16x3" scheme of Henry, Tang & Heinecke 2019):
//
//   half-transform  X[(Q,m)][j] = sum_n B_Q[m][n] U[n][j]   A = B slices, rows (Q,m), K-major
//                                                          B = U^T slices, rows j,   K-major
//   contraction     K[m][n] = sum_{Q,j} s_j X[m][Q,j] X[n][Q,j]   lower 128x128 tiles, split-K
//
// The B operand of the half-transform (dense, both triangles, BF16 hi/lo) is built once from
// the FP64 tiles.  Every operand lives in HBM pre-swizzled, in contiguous blocks that are the
// exact shared-memory image of one 64-byte-swizzled K-major tile (128 or 64 rows x 32 k), so
// the producer moves each tile with a single cp.async.bulk (TMA bulk copy) into a multi-stage
// ring guarded by mbarriers; the transform's epilogue writes X in that same blocked form.
// One thread issues tcgen05.mma; four warps drain the TMEM accumulators with tcgen05.ld.  The negative k-blocks of an incremental
// build use the instruction's negate-A bit.  Split-K partials (FP32) are summed in FP64 in
// a fixed order, so repeated builds are bitwise identical.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "block_lists.h"
#include "gdfjk.h"
#include "mixed.cuh"
#include "tc_common.cuh"

namespace gdfjk {

constexpr int MM = 128;                    // tile rows (MMA M)
constexpr int MK = tc::SWZ / 2;            // k per pipeline stage: one swizzle row of bf16
constexpr int A_TILE_BYTES = MM * MK * 2;  // 8 KB
constexpr int CN = 256;                    // contraction tile columns (MMA N)
constexpr int SMEM_BUDGET = 224 * 1024;
constexpr int SMEM_RESERVE = 2048;         // alignment slack + barriers

enum { MODE_TRANSFORM = 0, MODE_CONTRACT = 1 };

struct TcArgs {
    int nbf_p;        // padded nbf (multiple of 128)
    int nu_pad;       // columns of U (multiple of 64)
    int npos_pad;     // positive columns (multiple of 32)
    int n_mtiles;     // transform: 128-row tiles in total
    int n_cols;       // accumulator columns of this launch (transform) or 128 (contraction)
    int n_off;        // first U column of this launch (transform)
    unsigned long long kdim;  // naux * nu_pad
    __nv_bfloat16* Xhi;
    __nv_bfloat16* Xlo;
    int ntr;           // tile rows (nbf_p / 128)
    int kb_per_split;  // 32-wide k blocks per split
    int nkb_total;
    int ntiles_out;
    float* part;
    int stages;
    int tmem_cols;
    const int2* tiles;  // contraction: (row block of 128, column block of 256) covering the lower triangle
    const __nv_bfloat16* zero_blk;  // 8 KB of zeros (operand rows past the end)
    const __nv_bfloat16* Bsh;       // transform operands, pre-swizzled blocks
    const __nv_bfloat16* Bsl;
    const __nv_bfloat16* Uth;
    const __nv_bfloat16* Utl;
    int n_items;  // work items of this launch
    int nbuf;     // TMEM accumulators (2 overlaps the epilogue with the next item)
    int* err;
    // transform: the listed k blocks of each 128-row block (blocks of B that touch a stored
    // tile), mb_kb[mb_ptr[mb] .. mb_ptr[mb+1]); the split copy of B holds only those
    const int* mb_ptr;
    const int* mb_kb;
    int nnz, nmb;
    // extents in elements (checked in the bounds-checked build)
    size_t lim_Bs, lim_Ut, lim_X, lim_part;
};

__device__ __forceinline__ uint32_t pack_bf162(float a, float b) {
    __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
    return *reinterpret_cast<uint32_t*>(&v);
}

// Persistent, warp-specialised GEMM: one CTA per SM walks the work items (round robin).
// warp 0 lane 0: TMA producer over a ring of `stages` shared-memory stages;
// warp 1 lane 0: tcgen05.mma issuer into one of `nbuf` TMEM accumulators;
// warps 2-5:     epilogue (tcgen05.ld of the accumulator, then global stores), which
//                overlaps the MMAs of the next item when nbuf == 2.
constexpr int TC_THREADS = 192;

template <int MODE>
__device__ __forceinline__ void work_item(const TcArgs& a, int item, int& a_row, int& b_row, int& kb0, int& nkb,
                                          int& tile, int& split) {
    if (MODE == MODE_TRANSFORM) {
        a_row = item * MM;
        b_row = a.n_off;
        const int mb = item % a.nmb;
        kb0 = a.mb_ptr[mb];                  // first list entry of this row block
        nkb = a.mb_ptr[mb + 1] - kb0;        // listed k blocks
        tile = item;
        split = 0;
    } else {
        split = item / a.ntiles_out;  // split-major: concurrent CTAs share one k window in L2
        tile = item % a.ntiles_out;
        int2 ij = a.tiles[tile];
        a_row = ij.x * MM;
        b_row = ij.y * CN;
        kb0 = split * a.kb_per_split;
        nkb = min(a.kb_per_split, a.nkb_total - kb0);
    }
}

template <int MODE>
__global__ void __launch_bounds__(TC_THREADS, 1) tc_gemm_kernel(const TcArgs a) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int N = a.n_cols;
    const int b_bytes = N * MK * 2;
    const int a_bytes = 2 * A_TILE_BYTES;  // hi/lo of the A tile
    const int stage_bytes = a_bytes + 2 * b_bytes;
    uint64_t* full = reinterpret_cast<uint64_t*>(smem + (size_t)a.stages * stage_bytes);
    uint64_t* empty = full + a.stages;
    uint64_t* tfull = empty + a.stages;  // [2]
    uint64_t* tempty = tfull + 2;        // [2]
    uint32_t* tmem_holder = reinterpret_cast<uint32_t*>(tempty + 2);
    volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_holder + 1);

    const int warp = threadIdx.x / 32;
    const int nbuf = a.nbuf;
    if (threadIdx.x == 0) {
        for (int s = 0; s < a.stages; ++s) {
            tc::mbar_init(&full[s], 1);
            tc::mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&tfull[b], 1);
            tc::mbar_init(&tempty[b], 4);
        }
        *abort_flag = 0;
        tc::fence_barrier_init();
    }
    if (warp == 0) tc::tmem_alloc(tmem_holder, (uint32_t)a.tmem_cols);
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = *tmem_holder;

    if (threadIdx.x == 0) {
        // ---- producer: one bulk copy per operand slice per stage; stage/phase kept incrementally
        int s = 0;
        uint32_t ph = 0;
        long kg = 0;
        const size_t blkA = (size_t)MM * MK;  // elements per 128-row operand block
        for (int item = blockIdx.x; item < a.n_items && !*abort_flag; item += gridDim.x) {
            int a_row, b_row, kb0, nkb, tile, split;
            work_item<MODE>(a, item, a_row, b_row, kb0, nkb, tile, split);
            const __nv_bfloat16 *pah, *pal, *pbh, *pbl, *pch = nullptr, *pcl = nullptr;
            size_t stepb;
            if (MODE == MODE_TRANSFORM) {
                const size_t Q = (size_t)item / a.nmb;
                pah = a.Bsh + (Q * a.nnz + kb0) * blkA;  // the listed blocks of this row block, in order
                pal = a.Bsl + (Q * a.nnz + kb0) * blkA;
                pbh = a.Uth + (size_t)b_row * MK;        // + kb * nu_pad * MK per listed k block
                pbl = a.Utl + (size_t)b_row * MK;
                stepb = (size_t)a.nu_pad * MK;
            } else {
                const size_t nkbt = a.kdim / MK;
                pah = a.Xhi + ((size_t)(a_row / MM) * nkbt + kb0) * blkA;
                pal = a.Xlo + ((size_t)(a_row / MM) * nkbt + kb0) * blkA;
                const int rb0 = b_row / MM, nrb = a.nbf_p / MM;
                // the two 128-row halves of the 256-row B tile; rows past the end read zeros
                pbh = rb0 < nrb ? a.Xhi + ((size_t)rb0 * nkbt + kb0) * blkA : a.zero_blk;
                pbl = rb0 < nrb ? a.Xlo + ((size_t)rb0 * nkbt + kb0) * blkA : a.zero_blk;
                pch = rb0 + 1 < nrb ? a.Xhi + ((size_t)(rb0 + 1) * nkbt + kb0) * blkA : a.zero_blk;
                pcl = rb0 + 1 < nrb ? a.Xlo + ((size_t)(rb0 + 1) * nkbt + kb0) * blkA : a.zero_blk;
                stepb = blkA;
            }
            const size_t stepc0 = (MODE == MODE_CONTRACT && (b_row / MM) < a.nbf_p / MM) ? blkA : 0;
            const size_t stepc1 = (MODE == MODE_CONTRACT && (b_row / MM) + 1 < a.nbf_p / MM) ? blkA : 0;
            for (int kb = 0; kb < nkb; ++kb, ++kg) {
                if (kg >= a.stages && !tc::mbar_wait(&empty[s], ph ^ 1u, abort_flag, a.err)) break;
                bool in_range = true;
                if (MODE == MODE_TRANSFORM)
                    in_range = BCHK(kb0 + kb < a.nnz, a.err, BC_MX_A, kb0 + kb, a.nnz) &&
                               BRANGE(pah - a.Bsh, blkA, a.lim_Bs, a.err, BC_MX_A) &&
                               BRANGE((pbh - a.Uth) + (size_t)a.mb_kb[kb0 + kb] * stepb, (size_t)N * MK, a.lim_Ut, a.err,
                                      BC_MX_B);
                else
                    in_range = BRANGE(pah - a.Xhi, blkA, a.lim_X, a.err, BC_MX_A) &&
                               (stepc0 == 0 || BRANGE(pbh - a.Xhi, blkA, a.lim_X, a.err, BC_MX_B)) &&
                               (stepc1 == 0 || BRANGE(pch - a.Xhi, blkA, a.lim_X, a.err, BC_MX_B));
                if (!in_range) {
                    *abort_flag = 1;  // the consumers leave their waits; no copy of this stage was issued
                    break;
                }
                uint8_t* st = smem + (size_t)s * stage_bytes;
                tc::mbar_arrive_expect_tx(&full[s], (uint32_t)stage_bytes);
                tc::bulk_load(st, pah, A_TILE_BYTES, &full[s]);
                tc::bulk_load(st + A_TILE_BYTES, pal, A_TILE_BYTES, &full[s]);
                pah += blkA;
                pal += blkA;
                if (MODE == MODE_TRANSFORM) {
                    const size_t kof = (size_t)a.mb_kb[kb0 + kb] * stepb;
                    tc::bulk_load(st + a_bytes, pbh + kof, (uint32_t)b_bytes, &full[s]);
                    tc::bulk_load(st + a_bytes + b_bytes, pbl + kof, (uint32_t)b_bytes, &full[s]);
                } else {
                    tc::bulk_load(st + a_bytes, pbh, A_TILE_BYTES, &full[s]);
                    tc::bulk_load(st + a_bytes + A_TILE_BYTES, pch, A_TILE_BYTES, &full[s]);
                    tc::bulk_load(st + a_bytes + b_bytes, pbl, A_TILE_BYTES, &full[s]);
                    tc::bulk_load(st + a_bytes + b_bytes + A_TILE_BYTES, pcl, A_TILE_BYTES, &full[s]);
                    pbh += stepc0;
                    pbl += stepc0;
                    pch += stepc1;
                    pcl += stepc1;
                }
                if (++s == a.stages) {
                    s = 0;
                    ph ^= 1u;
                }
            }
        }
    } else if (threadIdx.x == 32) {
        // ---- MMA issuer: descriptors built once per stage and advanced by constants along k
        int s = 0;
        uint32_t ph = 0;
        int it = 0;
        const uint32_t smem_base = tc::smem_u32(smem);
        const int n1 = N < 256 ? N : 256;
        const int n2 = N - n1;  // second MMA of a row when N > 256
        const uint32_t id1p = tc::idesc_bf16_f32(MM, n1, false), id1n = tc::idesc_bf16_f32(MM, n1, true);
        const uint32_t id2p = n2 > 0 ? tc::idesc_bf16_f32(MM, n2, false) : 0u;
        const uint32_t id2n = n2 > 0 ? tc::idesc_bf16_f32(MM, n2, true) : 0u;
        const uint64_t boff2 = (uint64_t)((256 * MK * 2) >> 4);  // second N chunk inside the B tile
        for (int item = blockIdx.x; item < a.n_items && !*abort_flag; item += gridDim.x, ++it) {
            int a_row, b_row, kb0, nkb, tile, split;
            work_item<MODE>(a, item, a_row, b_row, kb0, nkb, tile, split);
            const int buf = it % nbuf, use = it / nbuf;
            if (use > 0 && !tc::mbar_wait(&tempty[buf], (uint32_t)((use - 1) & 1), abort_flag, a.err)) break;
            tc::tc_fence_after();
            const uint32_t d1 = tmem + (uint32_t)(buf * N), d2 = d1 + 256u;
            // position of the first k block inside its group of nu_pad columns (sign of dD)
            int kmod = (MODE == MODE_CONTRACT) ? (int)(((unsigned long long)kb0 * MK) % (unsigned long long)a.nu_pad) : 0;
            bool ok = true;
            for (int kb = 0; kb < nkb; ++kb) {
                if (!tc::mbar_wait(&full[s], ph, abort_flag, a.err)) {
                    ok = false;
                    break;
                }
                tc::tc_fence_after();
                const uint32_t st = smem_base + (uint32_t)(s * stage_bytes);
                const uint64_t dAh = tc::sdesc_kmajor(st), dAl = tc::sdesc_kmajor(st + A_TILE_BYTES);
                const uint64_t dBh = tc::sdesc_kmajor(st + a_bytes), dBl = tc::sdesc_kmajor(st + a_bytes + b_bytes);
                bool neg = false;
                if (MODE == MODE_CONTRACT) {
                    neg = kmod >= a.npos_pad;
                    kmod += MK;
                    if (kmod >= a.nu_pad) kmod -= a.nu_pad;
                }
                const uint32_t i1 = neg ? id1n : id1p, i2 = neg ? id2n : id2p;
#pragma unroll
                for (int ks = 0; ks < MK / 16; ++ks) {
                    const uint64_t ko = (uint64_t)(2 * ks);  // 32 bytes along k, in 16-byte units
                    const uint32_t acc0 = (kb | ks) != 0 ? 1u : 0u;
                    // hi*hi, hi*lo, lo*hi
                    tc::mma_bf16(d1, dAh + ko, dBh + ko, i1, acc0);
                    if (n2 > 0) tc::mma_bf16(d2, dAh + ko, dBh + ko + boff2, i2, acc0);
                    tc::mma_bf16(d1, dAh + ko, dBl + ko, i1, 1u);
                    if (n2 > 0) tc::mma_bf16(d2, dAh + ko, dBl + ko + boff2, i2, 1u);
                    tc::mma_bf16(d1, dAl + ko, dBh + ko, i1, 1u);
                    if (n2 > 0) tc::mma_bf16(d2, dAl + ko, dBh + ko + boff2, i2, 1u);
                }
                tc::mma_commit(&empty[s]);
                if (++s == a.stages) {
                    s = 0;
                    ph ^= 1u;
                }
            }
            tc::mma_commit(&tfull[buf]);
            if (!ok) break;
        }
    } else if (warp >= 2) {
        // ---- epilogue
        const int r = (warp % 4) * 32 + (threadIdx.x % 32);
        const uint32_t lane_base = tmem + ((uint32_t)((warp % 4) * 32) << 16);
        int it = 0;
        for (int item = blockIdx.x; item < a.n_items; item += gridDim.x, ++it) {
            int a_row, b_row, kb0, nkb, tile, split;
            work_item<MODE>(a, item, a_row, b_row, kb0, nkb, tile, split);
            const int buf = it % nbuf, use = it / nbuf;
            bool ok = tc::mbar_wait(&tfull[buf], (uint32_t)(use & 1), abort_flag, a.err);
            __syncwarp();
            if (!ok || *abort_flag) break;
            tc::tc_fence_after();
            const uint32_t cbase = lane_base + (uint32_t)(buf * N);
            if (MODE == MODE_TRANSFORM) {
                size_t grow = (size_t)a_row + r;
                size_t Q = grow / a.nbf_p, m = grow % a.nbf_p;
                // X goes out pre-swizzled in 8 KB blocks (128 rows x 32 k): exactly the
                // shared-memory image of one contraction operand tile
                const size_t nkbt = a.kdim / MK;
                const size_t rowblk = (m / MM) * nkbt;
                const uint32_t rr = (uint32_t)(m % MM);
                for (int c0 = 0; c0 < N; c0 += 16) {
                    uint32_t v[16];
                    tc::tmem_ld16(cbase + (uint32_t)c0, v);
                    uint32_t hi[8], lo[8];
#pragma unroll
                    for (int j = 0; j < 8; ++j) {
                        float x0 = __uint_as_float(v[2 * j]), x1 = __uint_as_float(v[2 * j + 1]);
                        __nv_bfloat16 h0 = __float2bfloat16_rn(x0), h1 = __float2bfloat16_rn(x1);
                        hi[j] = pack_bf162(__bfloat162float(h0), __bfloat162float(h1));
                        lo[j] = pack_bf162(x0 - __bfloat162float(h0), x1 - __bfloat162float(h1));
                    }
                    size_t k0 = Q * a.nu_pad + a.n_off + c0;
                    size_t blk = (rowblk + k0 / MK) * (size_t)(MM * MK);  // elements
                    uint32_t ch = (uint32_t)((k0 % MK) / 8);
                    uint32_t o0 = tc::swz_offset(rr, ch) / 2, o1 = tc::swz_offset(rr, ch + 1) / 2;
                    if (!BRANGE(blk, (size_t)MM * MK, a.lim_X, a.err, BC_MX_OUT)) continue;
                    *reinterpret_cast<uint4*>(a.Xhi + blk + o0) = make_uint4(hi[0], hi[1], hi[2], hi[3]);
                    *reinterpret_cast<uint4*>(a.Xhi + blk + o1) = make_uint4(hi[4], hi[5], hi[6], hi[7]);
                    *reinterpret_cast<uint4*>(a.Xlo + blk + o0) = make_uint4(lo[0], lo[1], lo[2], lo[3]);
                    *reinterpret_cast<uint4*>(a.Xlo + blk + o1) = make_uint4(lo[4], lo[5], lo[6], lo[7]);
                }
            } else {
                float* dst = a.part + (((size_t)split * a.ntiles_out + tile) * MM + r) * CN;
                const bool wok = BRANGE(dst - a.part, CN, a.lim_part, a.err, BC_MX_OUT);
                for (int c0 = 0; c0 < CN; c0 += 16) {
                    uint32_t v[16];
                    tc::tmem_ld16(cbase + (uint32_t)c0, v);  // warp-collective: every lane loads
                    if (!wok) continue;
                    float4* d4 = reinterpret_cast<float4*>(dst + c0);
#pragma unroll
                    for (int j = 0; j < 4; ++j)
                        d4[j] = make_float4(__uint_as_float(v[4 * j]), __uint_as_float(v[4 * j + 1]),
                                            __uint_as_float(v[4 * j + 2]), __uint_as_float(v[4 * j + 3]));
                }
            }
            tc::tc_fence_before();
            __syncwarp();
            if ((threadIdx.x % 32) == 0) tc::mbar_arrive(&tempty[buf]);
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
    if (warp == 0) tc::tmem_dealloc(tmem, (uint32_t)a.tmem_cols);
}

// ---------------------------------------------------------------- helper kernels
// BF16 hi/lo slices of B (both triangles) from the FP64 tiles, rows (Q, m), for the listed
// 128 x 32 blocks only (those that touch a stored tile): block (Q, entry) at
// (Q * nnz + entry) * 4096 elements, pre-swizzled.  One CUDA block per row (Q, m).
__global__ void split_B_kernel(const double* __restrict__ B, int naux, int nbf, int nT, int ntiles,
                               const int* __restrict__ map, int nbf_p, const int* __restrict__ mb_ptr,
                               const int* __restrict__ mb_kb, int nnz, __nv_bfloat16* __restrict__ Bh,
                               __nv_bfloat16* __restrict__ Bl) {
    size_t row = blockIdx.x;  // Q * nbf_p + m
    int Q = (int)(row / nbf_p), m = (int)(row % nbf_p);
    const int mb = m / MM, p0 = mb_ptr[mb], cnt = mb_ptr[mb + 1] - p0;
    for (int e = threadIdx.x; e < cnt * MK; e += blockDim.x) {
        const int p = e / MK, c = e % MK;
        const int n = mb_kb[p0 + p] * MK + c;
        double v = 0.0;
        if (m < nbf && n < nbf) {
            int I = m / TILE, J = n / TILE;
            int hi = I >= J ? I : J, lo = I >= J ? J : I;
            int t = map[hi * nT + lo];
            if (t >= 0) {
                size_t base = ((size_t)Q * ntiles + t) * TILE_ELEMS;
                v = (I >= J) ? B[base + (m % TILE) * TILE + (n % TILE)] : B[base + (n % TILE) * TILE + (m % TILE)];
            }
        }
        __nv_bfloat16 h = __double2bfloat16(v);
        // pre-swizzled 8 KB blocks (128 rows x 32 k): the shared-memory image of an operand tile
        size_t blk = ((size_t)Q * nnz + p0 + p) * (MM * MK);
        size_t off = blk + tc::swz_offset((uint32_t)(m % MM), (uint32_t)(c / 8)) / 2 + (c % 8);
        Bh[off] = h;
        Bl[off] = __double2bfloat16(v - (double)__bfloat162float(h));
    }
}

// U^T slices: row j < npos_pad holds column j of the positive group, row npos_pad + j holds
// column npos + j (negative group); padding rows/columns are zero.
__global__ void split_Ut_kernel(const double* __restrict__ U, int ldu, int nbf, int npos, int nneg, int npos_pad,
                                int nu_pad, int nbf_p, __nv_bfloat16* __restrict__ Uh, __nv_bfloat16* __restrict__ Ul) {
    size_t n = (size_t)nu_pad * nbf_p;
    for (size_t e = blockIdx.x * (size_t)blockDim.x + threadIdx.x; e < n; e += (size_t)gridDim.x * blockDim.x) {
        int j = (int)(e / nbf_p), k = (int)(e % nbf_p);
        int col = -1;
        if (j < npos_pad) {
            if (j < npos) col = j;
        } else if (j - npos_pad < nneg) {
            col = npos + (j - npos_pad);
        }
        double v = (col >= 0 && k < nbf) ? U[(size_t)k * ldu + col] : 0.0;
        __nv_bfloat16 h = __double2bfloat16(v);
        // k-block-major and pre-swizzled: all nu_pad rows of one 32-wide k block are contiguous,
        // so a stage's whole U^T operand is one bulk copy
        size_t off = (size_t)(k / MK) * ((size_t)nu_pad * MK) + tc::swz_offset((uint32_t)j, (uint32_t)((k % MK) / 8)) / 2 +
                     (k % 8);
        Uh[off] = h;
        Ul[off] = __double2bfloat16(v - (double)__bfloat162float(h));
    }
}

// K[m][n] (and its mirror), m >= n, = sum over splits (fixed order, FP64) of the partial
// tiles; `tile_of_block[I * ncb + Jc]` maps a (row block, column block) to its tile index.
__global__ void reduce_mixed_kernel(const float* __restrict__ part, int nsplit, int ntiles_out, int nbf,
                                    const int* __restrict__ tile_of_block, int ncb, double* __restrict__ K, int ldk,
                                    double* __restrict__ Kacc, int accumulate, size_t lim_part,
                                    int* __restrict__ err) {
    size_t n_lower = (size_t)nbf * (nbf + 1) / 2;
    for (size_t p = blockIdx.x * (size_t)blockDim.x + threadIdx.x; p < n_lower; p += (size_t)gridDim.x * blockDim.x) {
        size_t m = (size_t)((sqrt(8.0 * (double)p + 1.0) - 1.0) * 0.5);
        while (m * (m + 1) / 2 > p) --m;
        while ((m + 1) * (m + 2) / 2 <= p) ++m;
        size_t n = p - m * (m + 1) / 2;
        int I = (int)(m / MM), Jc = (int)(n / CN);
        int t = tile_of_block[I * ncb + Jc];
        size_t off = ((size_t)t * MM + (m % MM)) * CN + (n % CN);
        if (!BCHK(t >= 0, err, BC_RED, t, ntiles_out) ||
            !BRANGE((size_t)(nsplit - 1) * ntiles_out * MM * CN + off, 1, lim_part, err, BC_RED))
            continue;
        double s = 0.0;
        for (int k = 0; k < nsplit; ++k) s += (double)part[(size_t)k * ntiles_out * MM * CN + off];
        if (accumulate) s += Kacc[m * nbf + n];
        if (Kacc) {
            Kacc[m * nbf + n] = s;
            Kacc[n * nbf + m] = s;
        }
        K[m * ldk + n] = s;
        K[n * ldk + m] = s;
    }
}

// ---------------------------------------------------------------- host side
namespace {

int pow2_cols(int n) {
    int c = 32;
    while (c < n) c <<= 1;
    return c;
}

}  // namespace

struct MixedState {
    int nbf_p = 0;
    __nv_bfloat16 *Bh = nullptr, *Bl = nullptr;  // naux*nbf_p x nbf_p
    bool B_ready = false;
    __nv_bfloat16 *Uh = nullptr, *Ul = nullptr;
    size_t U_cap = 0;
    __nv_bfloat16 *Xh = nullptr, *Xl = nullptr;
    size_t X_cap = 0;
    float* part = nullptr;
    size_t part_cap = 0;
    double* Kacc = nullptr;  // running K of incremental builds (nbf x nbf)
    size_t Kacc_cap = 0;
    bool have_prev = false;
    int* err = nullptr;
    bool attrs_set = false;
    int num_sms = 0;
    int2* d_tiles = nullptr;
    int* d_tile_of_block = nullptr;
    int tiles_nbf_p = 0, ntiles_c = 0, ncb = 0;
    __nv_bfloat16* zero_blk = nullptr;
    int* d_mb_ptr = nullptr;  // listed blocks of B (block_lists.h)
    int* d_mb_kb = nullptr;
    int nnz = 0, lists_nbf_p = 0;
};

MixedState* mixed_create() { return new MixedState(); }

static void free_all(MixedState* m) {
    void* ps[] = {m->Bh, m->Bl, m->Uh, m->Ul, m->Xh, m->Xl, m->part, m->Kacc, m->err, m->d_tiles, m->d_tile_of_block,
                  m->zero_blk, m->d_mb_ptr, m->d_mb_kb};
    for (void* p : ps) big_free(p);
    m->Bh = m->Bl = m->Uh = m->Ul = m->Xh = m->Xl = nullptr;
    m->part = nullptr;
    m->Kacc = nullptr;
    m->err = nullptr;
    m->d_tiles = nullptr;
    m->d_tile_of_block = nullptr;
    m->zero_blk = nullptr;
    m->d_mb_ptr = m->d_mb_kb = nullptr;
    m->lists_nbf_p = 0;
    m->tiles_nbf_p = 0;
    m->U_cap = m->X_cap = m->part_cap = m->Kacc_cap = 0;
    m->B_ready = false;
    m->have_prev = false;
}

void mixed_destroy(MixedState* m) {
    if (!m) return;
    free_all(m);
    delete m;
}

void mixed_release(MixedState* m) {
    if (!m) return;
    void* ps[] = {m->Bh, m->Bl, m->Uh, m->Ul, m->Xh, m->Xl, m->part};
    for (void* p : ps) big_free(p);
    m->Bh = m->Bl = m->Uh = m->Ul = m->Xh = m->Xl = nullptr;
    m->part = nullptr;
    m->U_cap = m->X_cap = m->part_cap = 0;
    m->B_ready = false;
}

void mixed_invalidate(MixedState* m) {
    if (!m) return;
    mixed_release(m);
    m->have_prev = false;
}

size_t mixed_query_memory(int nbf, int naux, int max_nocc) {
    size_t nbf_p = (size_t)round_up(nbf, MM);
    size_t nu = (size_t)round_up(std::max(1, 2 * max_nocc), 64) + 64;
    size_t b = 2 * 2 * (size_t)naux * nbf_p * nbf_p;  // B slices
    b += 2 * 2 * nbf_p * naux * nu;                   // X slices
    b += 2 * 2 * nu * nbf_p + nbf_p * nbf_p * 8;
    return b;
}

static int dalloc_bytes(void** p, size_t bytes, std::string& err) {
    big_free(*p);
    *p = nullptr;
    cudaError_t e = engine_malloc(p, bytes);
    if (e != cudaSuccess) {
        cudaGetLastError();
        err = "mixed: device allocation of " + std::to_string(bytes / 1e9) + " GB refused";
        return GDFJK_ERR_OOM;
    }
    return GDFJK_OK;
}

// K_inc (written into K, nbf x nbf) = sum_Q B_Q (U+ U+^T - U- U-^T) B_Q; if `accumulate`,
// the running K is added and updated.
int mixed_k_factor(MixedState* m, const double* B, const TileLayout& L, const int* map_host, int nbf, int naux,
                   const double* U, int ldu, int npos, int nneg, int accumulate, double* K, cudaEvent_t ev_transform_done,
                   cudaStream_t s, std::string& err) {
    int rc;
    const int nbf_p = round_up(nbf, MM);
    if (!m->err) {
        if ((rc = dalloc_bytes((void**)&m->err, sizeof(int), err))) return rc;
        cudaMemsetAsync(m->err, 0, sizeof(int), s);
    }
    if (!m->zero_blk) {
        if ((rc = dalloc_bytes((void**)&m->zero_blk, A_TILE_BYTES, err))) return rc;
        cudaMemsetAsync(m->zero_blk, 0, A_TILE_BYTES, s);
    }
    if (m->lists_nbf_p != nbf_p) {
        const BlockLists bl = build_block_lists(map_host, L.nT, nbf_p, MM, MK, TILE);
        if (bl.kb.empty()) {
            err = "mixed: B has no stored tiles";
            return GDFJK_ERR_ARG;
        }
        if ((rc = dalloc_bytes((void**)&m->d_mb_ptr, bl.ptr.size() * sizeof(int), err)) ||
            (rc = dalloc_bytes((void**)&m->d_mb_kb, bl.kb.size() * sizeof(int), err)))
            return rc;
        cudaMemcpy(m->d_mb_ptr, bl.ptr.data(), bl.ptr.size() * sizeof(int), cudaMemcpyHostToDevice);
        cudaMemcpy(m->d_mb_kb, bl.kb.data(), bl.kb.size() * sizeof(int), cudaMemcpyHostToDevice);
        m->nnz = (int)bl.kb.size();
        m->lists_nbf_p = nbf_p;
        m->B_ready = false;
    }
    if (!m->B_ready || m->nbf_p != nbf_p) {
        size_t bytes = (size_t)naux * m->nnz * (MM * MK) * 2;
        m->B_ready = false;
        if ((rc = dalloc_bytes((void**)&m->Bh, bytes, err)) || (rc = dalloc_bytes((void**)&m->Bl, bytes, err))) return rc;
        split_B_kernel<<<(unsigned)((size_t)naux * nbf_p), 256, 0, s>>>(B, naux, nbf, L.nT, L.ntiles, L.map, nbf_p,
                                                                       m->d_mb_ptr, m->d_mb_kb, m->nnz, m->Bh, m->Bl);
        m->nbf_p = nbf_p;
        m->B_ready = true;
    }
    const int npos_pad = round_up(npos, MK);
    const int nneg_pad = round_up(nneg, MK);
    const int nu_pad = npos_pad + nneg_pad;
    if (nu_pad == 0) {
        cudaMemsetAsync(K, 0, sizeof(double) * (size_t)nbf * nbf, s);
        if (ev_transform_done) cudaEventRecord(ev_transform_done, s);
        return GDFJK_OK;
    }
    size_t ue = (size_t)nu_pad * nbf_p;
    if (ue > m->U_cap) {
        m->U_cap = 0;
        if ((rc = dalloc_bytes((void**)&m->Uh, ue * 2, err)) || (rc = dalloc_bytes((void**)&m->Ul, ue * 2, err))) return rc;
        m->U_cap = ue;
    }
    const unsigned long long kdim = (unsigned long long)naux * nu_pad;
    size_t xe = (size_t)nbf_p * kdim;
    if (xe > m->X_cap) {
        m->X_cap = 0;
        if ((rc = dalloc_bytes((void**)&m->Xh, xe * 2, err)) || (rc = dalloc_bytes((void**)&m->Xl, xe * 2, err))) return rc;
        m->X_cap = xe;
    }
    {
        int blocks = (int)std::min<size_t>((ue + 255) / 256, 152 * 16);
        split_Ut_kernel<<<blocks, 256, 0, s>>>(U, ldu, nbf, npos, nneg, npos_pad, nu_pad, nbf_p, m->Uh, m->Ul);
    }
    if (!m->num_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, dev);
        if (m->num_sms <= 0) m->num_sms = 152;
    }
    if (!m->attrs_set) {
        cudaFuncSetAttribute(tc_gemm_kernel<MODE_TRANSFORM>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BUDGET);
        cudaFuncSetAttribute(tc_gemm_kernel<MODE_CONTRACT>, cudaFuncAttributeMaxDynamicSharedMemorySize, SMEM_BUDGET);
        m->attrs_set = true;
    }
    // ---- half-transform, in accumulator chunks of at most 448 columns
    for (int n_off = 0; n_off < nu_pad; n_off += 448) {
        TcArgs ta{};
        ta.nbf_p = nbf_p;
        ta.nu_pad = nu_pad;
        ta.npos_pad = npos_pad;
        ta.n_cols = std::min(448, nu_pad - n_off);
        ta.n_off = n_off;
        ta.kdim = kdim;
        ta.Xhi = m->Xh;
        ta.Xlo = m->Xl;
        ta.err = m->err;
        ta.tiles = nullptr;
        ta.zero_blk = m->zero_blk;
        ta.Bsh = m->Bh;
        ta.Bsl = m->Bl;
        ta.Uth = m->Uh;
        ta.Utl = m->Ul;
        ta.mb_ptr = m->d_mb_ptr;
        ta.mb_kb = m->d_mb_kb;
        ta.nnz = m->nnz;
        ta.nmb = nbf_p / MM;
        // one 128-row tile per item; two TMEM accumulators when they fit, so the epilogue of one
        // item overlaps the MMAs of the next
        ta.n_mtiles = (int)((size_t)naux * nbf_p / MM);
        int stage_bytes = 2 * A_TILE_BYTES + 2 * ta.n_cols * MK * 2;
        ta.stages = std::min(8, (SMEM_BUDGET - SMEM_RESERVE) / stage_bytes);
        ta.nbuf = (2 * ta.n_cols <= 512) ? 2 : 1;
        ta.tmem_cols = pow2_cols(ta.nbuf * ta.n_cols);
        ta.n_items = ta.n_mtiles;
        ta.lim_Bs = (size_t)naux * m->nnz * (MM * MK);
        ta.lim_Ut = m->U_cap;
        ta.lim_X = m->X_cap;
        unsigned grid = (unsigned)std::min(ta.n_items, m->num_sms);
        tc_gemm_kernel<MODE_TRANSFORM><<<grid, TC_THREADS, SMEM_BUDGET, s>>>(ta);
    }
    if (ev_transform_done) cudaEventRecord(ev_transform_done, s);
    // ---- contraction: 128 x 256 tiles covering the lower triangle
    const int ntr = nbf_p / MM;
    if (m->tiles_nbf_p != nbf_p) {
        const int ncb = (nbf_p + CN - 1) / CN;
        std::vector<int2> tl;
        std::vector<int> tob((size_t)ntr * ncb, -1);
        for (int I = 0; I < ntr; ++I)
            for (int Jc = 0; Jc < ncb && Jc * CN <= I * MM + MM - 1; ++Jc) {
                tob[(size_t)I * ncb + Jc] = (int)tl.size();
                tl.push_back(make_int2(I, Jc));
            }
        if ((rc = dalloc_bytes((void**)&m->d_tiles, tl.size() * sizeof(int2), err)) ||
            (rc = dalloc_bytes((void**)&m->d_tile_of_block, tob.size() * sizeof(int), err)))
            return rc;
        cudaMemcpy(m->d_tiles, tl.data(), tl.size() * sizeof(int2), cudaMemcpyHostToDevice);
        cudaMemcpy(m->d_tile_of_block, tob.data(), tob.size() * sizeof(int), cudaMemcpyHostToDevice);
        m->ntiles_c = (int)tl.size();
        m->ncb = ncb;
        m->tiles_nbf_p = nbf_p;
    }
    const int ntiles_out = m->ntiles_c;
    const int nkb_total = (int)(kdim / MK);
    // at least ~8 work items per SM, and at most 256 k blocks (8192 terms) per FP32
    // accumulation run so the accumulation error stays below the BF16x3 splitting error
    int nsplit = std::max(1, (m->num_sms * 8 + ntiles_out - 1) / ntiles_out);
    nsplit = std::max(nsplit, (nkb_total + 255) / 256);
    nsplit = std::min(nsplit, std::max(1, nkb_total / 16));
    int kb_per_split = (nkb_total + nsplit - 1) / nsplit;
    nsplit = (nkb_total + kb_per_split - 1) / kb_per_split;
    size_t pe = (size_t)nsplit * ntiles_out * MM * CN;
    if (pe > m->part_cap) {
        m->part_cap = 0;
        if ((rc = dalloc_bytes((void**)&m->part, pe * 4, err))) return rc;
        m->part_cap = pe;
    }
    TcArgs ca{};
    ca.nbf_p = nbf_p;
    ca.nu_pad = nu_pad;
    ca.npos_pad = npos_pad;
    ca.n_cols = CN;
    ca.tiles = m->d_tiles;
    ca.zero_blk = m->zero_blk;
    ca.Xhi = m->Xh;
    ca.Xlo = m->Xl;
    ca.kdim = kdim;
    ca.ntr = ntr;
    ca.kb_per_split = kb_per_split;
    ca.nkb_total = nkb_total;
    ca.ntiles_out = ntiles_out;
    ca.part = m->part;
    ca.err = m->err;
    ca.stages = std::min(8, (SMEM_BUDGET - SMEM_RESERVE) / (2 * A_TILE_BYTES + 2 * CN * MK * 2));
    ca.nbuf = 2;
    ca.tmem_cols = pow2_cols(2 * CN);
    ca.n_items = ntiles_out * nsplit;
    ca.lim_X = m->X_cap;
    ca.lim_part = m->part_cap;
    unsigned cgrid = (unsigned)std::min(ca.n_items, m->num_sms);
    tc_gemm_kernel<MODE_CONTRACT><<<cgrid, TC_THREADS, SMEM_BUDGET, s>>>(ca);
    // ---- fixed-order FP64 reduction (+ running K for incremental builds)
    size_t kn = (size_t)nbf * nbf;
    if (kn > m->Kacc_cap) {
        m->Kacc_cap = 0;
        m->have_prev = false;
        if ((rc = dalloc_bytes((void**)&m->Kacc, kn * 8, err))) return rc;
        m->Kacc_cap = kn;
        m->have_prev = false;
    }
    int acc = (accumulate && m->have_prev) ? 1 : 0;
    {
        size_t nl = (size_t)nbf * (nbf + 1) / 2;
        int blocks = (int)std::min<size_t>((nl + 255) / 256, (size_t)m->num_sms * 16);
        reduce_mixed_kernel<<<blocks, 256, 0, s>>>(m->part, nsplit, ntiles_out, nbf, m->d_tile_of_block, m->ncb, K, nbf,
                                                   m->Kacc, acc, m->part_cap, m->err);
    }
    m->have_prev = true;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("mixed: launch failed: ") + cudaGetErrorString(e);
        return GDFJK_ERR_CUDA;
    }
    return GDFJK_OK;
}

namespace {
// The bounded wait of the tensor-core kernels (tc::mbar_wait) on an mbarrier that no thread
// and no copy ever arrives on: nothing is in flight, so the block simply returns once the
// wait has run out and raised its error bit.
__global__ void wait_probe_kernel(unsigned long long limit_ns, int* err) {
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort_flag;
    if (threadIdx.x == 0) {
        tc::mbar_init(&bar, 1);
        abort_flag = 0;
        tc::fence_barrier_init();
    }
    __syncthreads();
    if (threadIdx.x == 0) tc::mbar_wait(&bar, 0, &abort_flag, err, limit_ns);
}
}  // namespace

int mixed_wait_probe(MixedState* m, unsigned long long limit_ns, cudaStream_t s, std::string& err) {
    int rc;
    if (!m->err) {
        if ((rc = dalloc_bytes((void**)&m->err, sizeof(int), err))) return rc;
        cudaMemsetAsync(m->err, 0, sizeof(int), s);
    }
    wait_probe_kernel<<<1, 32, 0, s>>>(limit_ns, m->err);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        err = std::string("wait probe: launch failed: ") + cudaGetErrorString(e);
        return GDFJK_ERR_CUDA;
    }
    return GDFJK_OK;
}

int mixed_build_K(MixedState* m, const double* B, const TileLayout& L, const int* map_host, int nbf, int nbf_pad,
                  int naux, const double* Cpad, int nocc, int nocc_pad, int mode, double* K, cudaEvent_t ev_transform_done,
                  cudaStream_t stream, std::string& err) {
    (void)nbf_pad;
    (void)mode;
    // a full build: U = C_occ, all columns positive
    return mixed_k_factor(m, B, L, map_host, nbf, naux, Cpad, nocc_pad, nocc, 0, 0, K, ev_transform_done, stream, err);
}

int mixed_set_base(MixedState* m, const double* K, int nbf, cudaStream_t s, std::string& err) {
    size_t kn = (size_t)nbf * nbf;
    if (kn > m->Kacc_cap) {
        m->Kacc_cap = 0;
        m->have_prev = false;
        int rc = dalloc_bytes((void**)&m->Kacc, kn * 8, err);
        if (rc) return rc;
        m->Kacc_cap = kn;
    }
    if (cudaMemcpyAsync(m->Kacc, K, kn * 8, cudaMemcpyDeviceToDevice, s) != cudaSuccess) {
        err = "mixed: copying the FP64 base failed";
        return GDFJK_ERR_CUDA;
    }
    m->have_prev = true;
    return GDFJK_OK;
}

int mixed_error_flag(MixedState* m, cudaStream_t s) {
    if (!m || !m->err) return 0;
    int f = 0;
    cudaMemcpyAsync(&f, m->err, sizeof(int), cudaMemcpyDeviceToHost, s);
    cudaStreamSynchronize(s);
    if (f) cudaMemsetAsync(m->err, 0, sizeof(int), s);
    return f;
}

}  // namespace gdfjk
