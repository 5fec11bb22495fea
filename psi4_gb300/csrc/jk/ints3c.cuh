// ints3c.cuh — device code of the 3-index integrals and the metric (ints3c.cu): the
// McMurchie–Davidson class kernels, instantiated per fitting-shell angular momentum in
// ints3c_lc0.cu .. ints3c_lc4.cu.
#pragma once

#include <cuda_runtime.h>

#include "../ints/gto_tables.h"

namespace gdfjk {
namespace ints {

constexpr int MAXL_PAIR = 3;  // primary shells: up to f
constexpr int MAXL_FIT = 4;   // fitting shells: up to g (also the metric's row shells)
constexpr int BOYS_NMAX = 2 * MAXL_PAIR + MAXL_FIT + 1;  // + 1: first derivatives
constexpr int BOYS_STRIDE = BOYS_NMAX + gto::BOYS_KT + 1;
constexpr int ERI_THREADS = 64;

__host__ __device__ constexpr int ncart(int l) { return (l + 1) * (l + 2) / 2; }
__host__ __device__ constexpr int ntuv(int L) { return L < 0 ? 0 : (L + 1) * (L + 2) * (L + 3) / 6; }
// position of (t, u, v), t + u + v <= L, in lexicographic (t, u, v) order
__host__ __device__ constexpr int tuv_index(int L, int t, int u, int v) {
    return ntuv(L) - ntuv(L - t) + u * (L - t + 1) - u * (u - 1) / 2 + v;
}
// Cartesian component k of angular momentum l (order x^l, x^(l-1) y, x^(l-1) z, ...):
// k = n(n+1)/2 + z with n = l - x = y + z
__host__ __device__ constexpr int cart_n(int k) { return k < 1 ? 0 : k < 3 ? 1 : k < 6 ? 2 : k < 10 ? 3 : 4; }
__host__ __device__ constexpr int cart_x(int l, int k) { return l - cart_n(k); }
__host__ __device__ constexpr int cart_z(int k) { return k - cart_n(k) * (cart_n(k) + 1) / 2; }
__host__ __device__ constexpr int cart_y(int k) { return cart_n(k) - cart_z(k); }
__host__ __device__ constexpr int pure_off(int l) { return l == 0 ? 0 : l == 1 ? 1 : l == 2 ? 10 : l == 3 ? 40 : 110; }
constexpr int PURE_TABLE = 245;  // sum over l <= 4 of (2l+1) ncart(l)

struct Shells {
    const int* atom;  // atom of each shell (the gradients' centres)
    const int* l;
    const int* nprim;
    const int* poff;
    const int* foff;
    const double* xyz;
    const double* exps;
    const double* coefs;
};

struct Eri3Args {
    Shells ab;          // shells of the pairs (the primary basis; the fitting basis for the metric)
    Shells cs;          // fitting shells
    const int2* pairs;  // (shell of angular momentum LA, shell of LB); y < 0: the unit function at x's centre
    const int* fits;    // fitting shells of class LC
    int nfit;
    int pure_ab, pure_c;
    double* out;
    long long ldo;
    int p0, p1;
    const long long* col_map;  // column of packed pair m(m+1)/2+n, < 0: not stored (nullable)
    const double* boys;  // Boys grid
    const double* pure;  // Cartesian -> solid harmonic matrices, l = 0..4 at pure_off(l)
    int metric;          // 1: out[(P - p0) * ldo + Q]
};

// F_0..F_N(T)
template <int N>
__device__ __forceinline__ void boys(const double* __restrict__ tab, double T, double* F) {
    if (T < gto::BOYS_TMAX) {
        const int g = (int)(T * (1.0 / gto::BOYS_H) + 0.5);
        const double dT = g * gto::BOYS_H - T;  // F_N(T) = sum_k F_{N+k}(T_g) (T_g - T)^k / k!
        const double* row = tab + (size_t)g * BOYS_STRIDE + N;
        double f = 0.0, pw = 1.0;
#pragma unroll
        for (int k = 0; k < gto::BOYS_KT; ++k) {
            f = fma(__ldg(row + k), pw, f);
            pw *= dT * (1.0 / (k + 1));
        }
        F[N] = f;
        if (N > 0) {
            const double e = exp(-T);
#pragma unroll
            for (int m = N - 1; m >= 0; --m) F[m] = (2.0 * T * F[m + 1] + e) * (1.0 / (2 * m + 1));
        }
    } else {
        const double e = exp(-T);
        F[0] = 0.5 * sqrt(M_PI / T) * erf(sqrt(T));
#pragma unroll
        for (int m = 0; m < N; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) * (0.5 / T);
    }
}

// Loop forms.  A class is "small" when its Cartesian block and Hermite orders are small
// enough to live in registers: its loops are fully unrolled, and every loop bound is a
// constant with the triangular limits as guards that fold away once the outer indices are
// constants (an unroll pragma on a loop whose bound depends on an outer index would be
// unrolled as a runtime loop first, multiplying the code).  The other classes run plain
// loops with their arrays in local memory; they carry a small share of the work.

// Hermite Coulomb integrals R_tuv = R^0_tuv(alpha, X, Y, Z), t+u+v <= L, in place: the array
// holds order n+1 for t+u+v <= L-n-1 while order n overwrites sums L-n down to 1 (each entry
// of sum s reads sums s-1 and s-2 of order n+1, not yet overwritten), then R_000.
__device__ __forceinline__ double r_step(const double* R, int L, int t, int u, int v, double X, double Y, double Z) {
    double val;
    if (t > 0) {
        val = X * R[tuv_index(L, t - 1, u, v)];
        if (t > 1) val = fma((double)(t - 1), R[tuv_index(L, t - 2, u, v)], val);
    } else if (u > 0) {
        val = Y * R[tuv_index(L, 0, u - 1, v)];
        if (u > 1) val = fma((double)(u - 1), R[tuv_index(L, 0, u - 2, v)], val);
    } else {
        val = Z * R[tuv_index(L, 0, 0, v - 1)];
        if (v > 1) val = fma((double)(v - 1), R[tuv_index(L, 0, 0, v - 2)], val);
    }
    return val;
}

template <int L, bool SMALL>
__device__ __forceinline__ void hermite_r(double alpha, double X, double Y, double Z, const double* F, double* R) {
    double pw[L + 1];  // (-2 alpha)^n
    pw[0] = 1.0;
#pragma unroll
    for (int n = 1; n <= L; ++n) pw[n] = pw[n - 1] * (-2.0 * alpha);
    R[0] = pw[L] * F[L];
    if constexpr (SMALL) {
#pragma unroll
        for (int n = L - 1; n >= 0; --n) {
#pragma unroll
            for (int s = L; s >= 1; --s)
#pragma unroll
                for (int t = 0; t <= L; ++t)
#pragma unroll
                    for (int u = 0; u <= L; ++u)
                        if (s <= L - n && t <= s && u <= s - t)
                            R[tuv_index(L, t, u, s - t - u)] = r_step(R, L, t, u, s - t - u, X, Y, Z);
            R[0] = pw[n] * F[n];
        }
    } else {
#pragma unroll 1
        for (int n = L - 1; n >= 0; --n) {
#pragma unroll 1
            for (int s = L - n; s >= 1; --s)
#pragma unroll 1
                for (int t = 0; t <= s; ++t)
#pragma unroll 1
                    for (int u = 0; u <= s - t; ++u) R[tuv_index(L, t, u, s - t - u)] = r_step(R, L, t, u, s - t - u, X, Y, Z);
            R[0] = pw[n] * F[n];
        }
    }
}

// 1D Hermite coefficients of a primitive product (recurrences of eq. 9.5.6-9.5.7):
// E[(i * (LB+1) + j) * (LA+LB+1) + t], i <= LA, j <= LB, t <= i + j
template <int LA, int LB>
__device__ __forceinline__ void hermite_1d(double a, double b, double A, double B, double* E) {
    constexpr int T = LA + LB + 1;
    const double p = a + b, mu = a * b / p, P = (a * A + b * B) / p;
    const double XPA = P - A, XPB = P - B, XAB = A - B, o2p = 0.5 / p;
#pragma unroll
    for (int k = 0; k < (LA + 1) * (LB + 1) * T; ++k) E[k] = 0.0;
    E[0] = exp(-mu * XAB * XAB);
#pragma unroll
    for (int i = 0; i < LA; ++i)
#pragma unroll
        for (int t = 0; t < T; ++t)
            if (t <= i + 1) {
                double v = XPA * E[(i * (LB + 1)) * T + t];
                if (t > 0) v += o2p * E[(i * (LB + 1)) * T + t - 1];
                if (t + 1 <= i) v += (t + 1) * E[(i * (LB + 1)) * T + t + 1];
                E[((i + 1) * (LB + 1)) * T + t] = v;
            }
#pragma unroll
    for (int i = 0; i <= LA; ++i)
#pragma unroll
        for (int j = 0; j < LB; ++j)
#pragma unroll
            for (int t = 0; t < T; ++t)
                if (t <= i + j + 1) {
                    double v = XPB * E[(i * (LB + 1) + j) * T + t];
                    if (t > 0) v += o2p * E[(i * (LB + 1) + j) * T + t - 1];
                    if (t + 1 <= i + j) v += (t + 1) * E[(i * (LB + 1) + j) * T + t + 1];
                    E[(i * (LB + 1) + j + 1) * T + t] = v;
                }
}

// Cartesian -> solid harmonics of one index of a block: OUTER groups of stride SO, the
// component index of stride SI, INNER contiguous entries per component; in place, the pure
// components in the first 2l+1 slots.
template <int L, int OUTER, int SO, int SI, int INNER>
__device__ __forceinline__ void to_pure(const double* __restrict__ c_pure, double* blk) {
    constexpr int NC = ncart(L), NP = 2 * L + 1;
    if constexpr (L > 0) {
#pragma unroll 1
        for (int o = 0; o < OUTER; ++o)
#pragma unroll 1
            for (int i = 0; i < INNER; ++i) {
                double tmp[NP];
#pragma unroll
                for (int r = 0; r < NP; ++r) {
                    double s = 0.0;
#pragma unroll
                    for (int k = 0; k < NC; ++k) s = fma(__ldg(c_pure + pure_off(L) + r * NC + k), blk[o * SO + k * SI + i], s);
                    tmp[r] = s;
                }
#pragma unroll
                for (int r = 0; r < NP; ++r) blk[o * SO + r * SI + i] = tmp[r];
            }
    }
}
template <int L, int OUTER, int SO, int SI, int INNER>
__device__ __forceinline__ void to_pure_unrolled(const double* __restrict__ c_pure, double* blk) {
    constexpr int NC = ncart(L), NP = 2 * L + 1;
    if constexpr (L > 0) {
#pragma unroll
        for (int o = 0; o < OUTER; ++o)
#pragma unroll
            for (int i = 0; i < INNER; ++i) {
                double tmp[NP];
#pragma unroll
                for (int r = 0; r < NP; ++r) {
                    double s = 0.0;
#pragma unroll
                    for (int k = 0; k < NC; ++k) s = fma(__ldg(c_pure + pure_off(L) + r * NC + k), blk[o * SO + k * SI + i], s);
                    tmp[r] = s;
                }
#pragma unroll
                for (int r = 0; r < NP; ++r) blk[o * SO + r * SI + i] = tmp[r];
            }
    }
}

// W_tuv = sum over the fitting Gaussian's Hermite terms (tx, ty, tz) of component (cx, cy, cz)
// of Ec[cx][tx] Ec[cy][ty] Ec[cz][tz] R_{t+tx, u+ty, v+tz}, t+u+v <= LAB
template <int LAB, int LC, int L>
__device__ __forceinline__ void ket_sum_small(const double* Ec, const double* R, int cx, int cy, int cz, double* W) {
#pragma unroll
    for (int t = 0; t <= LAB; ++t)
#pragma unroll
        for (int u = 0; u <= LAB; ++u)
#pragma unroll
            for (int v = 0; v <= LAB; ++v)
                if (t + u + v <= LAB) {
                    double s = 0.0;
#pragma unroll
                    for (int tx = 0; tx <= LC; ++tx)
#pragma unroll
                        for (int ty = 0; ty <= LC; ++ty)
#pragma unroll
                            for (int tz = 0; tz <= LC; ++tz)
                                if (tx <= cx && ty <= cy && tz <= cz && !((cx - tx) & 1) && !((cy - ty) & 1) &&
                                    !((cz - tz) & 1))
                                    s = fma(Ec[cx * (LC + 1) + tx] * Ec[cy * (LC + 1) + ty] * Ec[cz * (LC + 1) + tz],
                                            R[tuv_index(L, t + tx, u + ty, v + tz)], s);
                    W[tuv_index(LAB, t, u, v)] = s;
                }
}
template <int LAB, int LC, int L>
__device__ __forceinline__ void ket_sum_loop(const double* Ec, const double* R, int cx, int cy, int cz, double* W) {
#pragma unroll 1
    for (int t = 0; t <= LAB; ++t)
#pragma unroll 1
        for (int u = 0; u <= LAB - t; ++u)
#pragma unroll 1
            for (int v = 0; v <= LAB - t - u; ++v) {
                double s = 0.0;
                for (int tx = cx & 1; tx <= cx; tx += 2)
                    for (int ty = cy & 1; ty <= cy; ty += 2)
                        for (int tz = cz & 1; tz <= cz; tz += 2)
                            s = fma(Ec[cx * (LC + 1) + tx] * Ec[cy * (LC + 1) + ty] * Ec[cz * (LC + 1) + tz],
                                    R[tuv_index(L, t + tx, u + ty, v + tz)], s);
                W[tuv_index(LAB, t, u, v)] = s;
            }
}

// sum_{t,u,v} Ex[t] Ey[u] Ez[v] W_tuv over t <= nx, u <= ny, v <= nz, one dimension at a time
template <int LAB>
__device__ __forceinline__ double bra_sum_small(const double* ex, const double* ey, const double* ez, int nx, int ny, int nz,
                                                const double* W) {
    double s = 0.0;
#pragma unroll
    for (int t = 0; t <= LAB; ++t)
        if (t <= nx) {
            double su = 0.0;
#pragma unroll
            for (int u = 0; u <= LAB; ++u)
                if (u <= ny && t + u <= LAB) {
                    double sv = 0.0;
#pragma unroll
                    for (int v = 0; v <= LAB; ++v)
                        if (v <= nz && t + u + v <= LAB) sv = fma(ez[v], W[tuv_index(LAB, t, u, v)], sv);
                    su = fma(ey[u], sv, su);
                }
            s = fma(ex[t], su, s);
        }
    return s;
}
template <int LAB>
__device__ __forceinline__ double bra_sum_loop(const double* ex, const double* ey, const double* ez, int nx, int ny, int nz,
                                               const double* W) {
    double s = 0.0;
#pragma unroll 1
    for (int t = 0; t <= nx; ++t) {
        double su = 0.0;
#pragma unroll 1
        for (int u = 0; u <= ny; ++u) {
            double sv = 0.0;
            for (int v = 0; v <= nz; ++v) sv = fma(ez[v], W[tuv_index(LAB, t, u, v)], sv);
            su = fma(ey[u], sv, su);
        }
        s = fma(ex[t], su, s);
    }
    return s;
}

template <int LA, int LB, int LC>
__global__ void __launch_bounds__(ERI_THREADS) eri3c_kernel(const Eri3Args a) {
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC);
    constexpr int LAB = LA + LB, L = LAB + LC;
    constexpr int NTAB = ntuv(LAB), NTL = ntuv(L);
    constexpr int TE = LAB + 1;
    constexpr int ED = (LA + 1) * (LB + 1) * TE;  // E entries of one dimension
    constexpr int PPW = 5 + 3 * ED;              // doubles per primitive product in shared memory
    constexpr bool SMALL = NA * NB * NC <= 36 && L <= 5;
    constexpr int UNR = SMALL ? 64 : 1;  // constant-bound loops over the block
    extern __shared__ double shp[];
    const int2 pr = a.pairs[blockIdx.x];
    const int sa = pr.x, sb = pr.y;
    const bool unit_b = sb < 0;
    const double* Ac = a.ab.xyz + 3 * sa;
    const double* Bc = unit_b ? Ac : a.ab.xyz + 3 * sb;
    const int npa = a.ab.nprim[sa], npb = unit_b ? 1 : a.ab.nprim[sb];
    const int npp = npa * npb;
    for (int k = threadIdx.x; k < npp; k += blockDim.x) {
        const int ia = k / npb, ib = k % npb;
        const double ea = a.ab.exps[a.ab.poff[sa] + ia];
        const double eb = unit_b ? 0.0 : a.ab.exps[a.ab.poff[sb] + ib];
        const double p = ea + eb;
        double* w = shp + (size_t)k * PPW;
        w[0] = p;
#pragma unroll
        for (int d = 0; d < 3; ++d) w[1 + d] = (ea * Ac[d] + eb * Bc[d]) / p;
        w[4] = a.ab.coefs[a.ab.poff[sa] + ia] * (unit_b ? 1.0 : a.ab.coefs[a.ab.poff[sb] + ib]);
#pragma unroll
        for (int d = 0; d < 3; ++d) hermite_1d<LA, LB>(ea, eb, Ac[d], Bc[d], w + 5 + d * ED);
    }
    __syncthreads();
    const int ci = blockIdx.y * blockDim.x + threadIdx.x;
    if (ci >= a.nfit) return;
    const int sc = a.fits[ci];
    const double* Cc = a.cs.xyz + 3 * sc;
    const int npc = a.cs.nprim[sc], pc0 = a.cs.poff[sc];
    double acc[NA * NB * NC];
#pragma unroll UNR
    for (int k = 0; k < NA * NB * NC; ++k) acc[k] = 0.0;
    constexpr double TWO_PI_52 = 34.986836655249725;  // 2 pi^(5/2)
    constexpr double SGN = (LC & 1) ? -1.0 : 1.0;      // (-1)^(tau+nu+phi): the ket's E vanish off parity LC
    for (int k = 0; k < npp; ++k) {
        const double* w = shp + (size_t)k * PPW;
        const double p = w[0];
        const double* Ex = w + 5;
        const double* Ey = w + 5 + ED;
        const double* Ez = w + 5 + 2 * ED;
        for (int kc = 0; kc < npc; ++kc) {
            const double c = a.cs.exps[pc0 + kc];
            const double pc = p + c, alpha = p * c / pc;
            const double X = w[1] - Cc[0], Y = w[2] - Cc[1], Z = w[3] - Cc[2];
            double F[L + 1];
            boys<L>(a.boys, alpha * (X * X + Y * Y + Z * Z), F);
            double R[NTL];
            hermite_r<L, SMALL>(alpha, X, Y, Z, F, R);
            const double pref = SGN * TWO_PI_52 / (p * c * sqrt(pc)) * w[4] * a.cs.coefs[pc0 + kc];
            // Hermite coefficients of the fitting Gaussian x^i exp(-c x^2): Ec[i][tau]
            double Ec[(LC + 1) * (LC + 1)];
#pragma unroll
            for (int q = 0; q < (LC + 1) * (LC + 1); ++q) Ec[q] = 0.0;
            Ec[0] = 1.0;
            const double o2c = 0.5 / c;
#pragma unroll
            for (int i = 0; i < LC; ++i)
#pragma unroll
                for (int t = 0; t <= LC; ++t)
                    if (t <= i + 1) {
                        double v = 0.0;
                        if (t > 0) v += o2c * Ec[i * (LC + 1) + t - 1];
                        if (t + 1 <= i) v += (t + 1) * Ec[i * (LC + 1) + t + 1];
                        Ec[(i + 1) * (LC + 1) + t] = v;
                    }
            if constexpr (SMALL) {
#pragma unroll
                for (int kq = 0; kq < NC; ++kq) {
                    double W[NTAB];
                    ket_sum_small<LAB, LC, L>(Ec, R, cart_x(LC, kq), cart_y(kq), cart_z(kq), W);
#pragma unroll
                    for (int ka = 0; ka < NA; ++ka)
#pragma unroll
                        for (int kb = 0; kb < NB; ++kb) {
                            const int ix = cart_x(LA, ka), iy = cart_y(ka), iz = cart_z(ka);
                            const int jx = cart_x(LB, kb), jy = cart_y(kb), jz = cart_z(kb);
                            const double s =
                                bra_sum_small<LAB>(Ex + (ix * (LB + 1) + jx) * TE, Ey + (iy * (LB + 1) + jy) * TE,
                                                   Ez + (iz * (LB + 1) + jz) * TE, ix + jx, iy + jy, iz + jz, W);
                            acc[(ka * NB + kb) * NC + kq] = fma(pref, s, acc[(ka * NB + kb) * NC + kq]);
                        }
                }
            } else {
#pragma unroll 1
                for (int kq = 0; kq < NC; ++kq) {
                    double W[NTAB];
                    ket_sum_loop<LAB, LC, L>(Ec, R, cart_x(LC, kq), cart_y(kq), cart_z(kq), W);
#pragma unroll 1
                    for (int ka = 0; ka < NA; ++ka)
#pragma unroll 1
                        for (int kb = 0; kb < NB; ++kb) {
                            const int ix = cart_x(LA, ka), iy = cart_y(ka), iz = cart_z(ka);
                            const int jx = cart_x(LB, kb), jy = cart_y(kb), jz = cart_z(kb);
                            const double s =
                                bra_sum_loop<LAB>(Ex + (ix * (LB + 1) + jx) * TE, Ey + (iy * (LB + 1) + jy) * TE,
                                                  Ez + (iz * (LB + 1) + jz) * TE, ix + jx, iy + jy, iz + jz, W);
                            acc[(ka * NB + kb) * NC + kq] = fma(pref, s, acc[(ka * NB + kb) * NC + kq]);
                        }
                }
            }
        }
    }
    // Cartesian -> solid harmonics (index of C, then B, then A), in place
    if constexpr (SMALL) {
        if (a.pure_c) to_pure_unrolled<LC, NA * NB, NC, 1, 1>(a.pure, acc);
        if (a.pure_ab) {
            to_pure_unrolled<LB, NA, NB * NC, NC, NC>(a.pure, acc);
            to_pure_unrolled<LA, 1, 0, NB * NC, NB * NC>(a.pure, acc);
        }
    } else {
        if (a.pure_c) to_pure<LC, NA * NB, NC, 1, 1>(a.pure, acc);
        if (a.pure_ab) {
            to_pure<LB, NA, NB * NC, NC, NC>(a.pure, acc);
            to_pure<LA, 1, 0, NB * NC, NB * NC>(a.pure, acc);
        }
    }
    const int na = a.pure_ab ? 2 * LA + 1 : NA, nb = unit_b ? 1 : (a.pure_ab ? 2 * LB + 1 : NB);
    const int nc = a.pure_c ? 2 * LC + 1 : NC;
    const int fa = a.ab.foff[sa], fb = unit_b ? 0 : a.ab.foff[sb], fc = a.cs.foff[sc];
    // the writes: guards on constant-bound loops keep the block's indices constant (registers)
#pragma unroll UNR
    for (int q = 0; q < NC; ++q) {
        const int P = fc + q;
        if (q >= nc || P < a.p0 || P >= a.p1) continue;
        double* row = a.out + (size_t)(P - a.p0) * a.ldo;
#pragma unroll UNR
        for (int ka = 0; ka < NA; ++ka) {
            if (ka >= na) continue;
            const long long m = fa + ka;
#pragma unroll UNR
            for (int kb = 0; kb < NB; ++kb) {
                if (kb >= nb) continue;
                const double v = acc[(ka * NB + kb) * NC + q];
                if (a.metric) {
                    row[m] = v;
                    continue;
                }
                const long long n = fb + kb;
                if (sa == sb && m < n) continue;  // diagonal shell pair: the lower triangle
                long long col = m >= n ? m * (m + 1) / 2 + n : n * (n + 1) / 2 + m;
                if (a.col_map) {
                    col = a.col_map[col];
                    if (col < 0) continue;
                }
                row[col] = v;
            }
        }
    }
}

// ---------------------------------------------------------------- first derivatives
// The gradient's contraction of the 3-index density with derivative integrals (psi4's
// DFJKGrad::build_Amn_x_terms, psi4/src/psi4/scfgrad/jk_grad.cc:868-1245, and the metric's
// MintsHelper::metric_grad, psi4/src/psi4/libmints/mintshelper.cc:2388):
//   grad[atom(A)] += sum G[P][mn] d(P|mn)/dA, grad[atom(B)] += ... d/dB,
//   grad[atom(C)] -= both (translational invariance), C the fitting shell.
// Derivatives of the Gaussians (d/dA_x x_A^i e^{-a x_A^2} = 2a x_A^(i+1) e^.. - i x_A^(i-1) e^..)
// fold into the pair's Hermite coefficients, so the Hermite sums run one order higher.  The
// density block is taken from solid harmonics to Cartesian components once per triplet and
// contracted on the fly: no derivative integral is stored.
struct Eri3GradArgs {
    Shells ab, cs;
    const int2* pairs;
    const int* fits;
    int nfit;
    int pure_ab, pure_c;
    const double* G;           // density rows: row P at G + P * ldg, columns as Eri3Args' out
    long long ldg;
    const long long* col_map;  // nullable
    double* grad;              // [natom][3], accumulated
    const double* boys;
    const double* pure;
    int metric;                // 1: G[P][Q] against (P|Q), the pair being (Q, unit)
    // point charges instead of fitting shells (nullable): fits index atoms with charge
    // charges[i] at charge_xyz[3i..]; the nuclear attraction -Z (mn|1/r_C) (lc = 0)
    const double* charges;
    const double* charge_xyz;
};

// adjoint of to_pure: pure components in the first 2l+1 slots of the index -> all ncart slots
template <int L, int OUTER, int SO, int SI, int INNER>
__device__ __forceinline__ void from_pure(const double* __restrict__ c_pure, double* blk) {
    constexpr int NC = ncart(L), NP = 2 * L + 1;
    if constexpr (L > 0) {
#pragma unroll 1
        for (int o = 0; o < OUTER; ++o)
#pragma unroll 1
            for (int i = 0; i < INNER; ++i) {
                double tmp[NC];
#pragma unroll
                for (int k = 0; k < NC; ++k) {
                    double s = 0.0;
#pragma unroll
                    for (int r = 0; r < NP; ++r) s = fma(__ldg(c_pure + pure_off(L) + r * NC + k), blk[o * SO + r * SI + i], s);
                    tmp[k] = s;
                }
#pragma unroll
                for (int k = 0; k < NC; ++k) blk[o * SO + k * SI + i] = tmp[k];
            }
    }
}

template <int LA, int LB, int LC>
__global__ void __launch_bounds__(ERI_THREADS) eri3c_grad_kernel(const Eri3GradArgs a) {
    constexpr int NA = ncart(LA), NB = ncart(LB), NC = ncart(LC);
    constexpr int LAB = LA + LB, LW = LAB + 1, L = LW + LC;
    constexpr int NTW = ntuv(LW), NTL = ntuv(L);
    constexpr int TE = LAB + 3;                  // t range of E with i <= LA+1, j <= LB+1
    constexpr int ED = (LA + 2) * (LB + 2) * TE;
    constexpr int PPW = 7 + 3 * ED;              // p, P, coefficient product, a, b, E tables
    extern __shared__ double shp[];
    __shared__ double red[6][ERI_THREADS];
    const int2 pr = a.pairs[blockIdx.x];
    const int sa = pr.x, sb = pr.y;
    const bool unit_b = sb < 0;
    const double* Ac = a.ab.xyz + 3 * sa;
    const double* Bc = unit_b ? Ac : a.ab.xyz + 3 * sb;
    const int npa = a.ab.nprim[sa], npb = unit_b ? 1 : a.ab.nprim[sb];
    const int npp = npa * npb;
    for (int k = threadIdx.x; k < npp; k += blockDim.x) {
        const int ia = k / npb, ib = k % npb;
        const double ea = a.ab.exps[a.ab.poff[sa] + ia];
        const double eb = unit_b ? 0.0 : a.ab.exps[a.ab.poff[sb] + ib];
        const double p = ea + eb;
        double* w = shp + (size_t)k * PPW;
        w[0] = p;
#pragma unroll
        for (int d = 0; d < 3; ++d) w[1 + d] = (ea * Ac[d] + eb * Bc[d]) / p;
        w[4] = a.ab.coefs[a.ab.poff[sa] + ia] * (unit_b ? 1.0 : a.ab.coefs[a.ab.poff[sb] + ib]);
        w[5] = ea;
        w[6] = eb;
#pragma unroll
        for (int d = 0; d < 3; ++d) hermite_1d<LA + 1, LB + 1>(ea, eb, Ac[d], Bc[d], w + 7 + d * ED);
    }
    __syncthreads();
    const int atomA = a.ab.atom[sa], atomB = unit_b ? atomA : a.ab.atom[sb];
    const int ci = blockIdx.y * blockDim.x + threadIdx.x;
    double gA[3] = {0.0, 0.0, 0.0}, gB[3] = {0.0, 0.0, 0.0};
    int atomC = -1;
    const bool point = a.charges != nullptr;
    if (ci < a.nfit) {
        const int sc = a.fits[ci];
        atomC = point ? sc : a.cs.atom[sc];
        if (!(atomA == atomB && atomB == atomC)) {
            // the density block in solid harmonics, then in Cartesian components
            double g[NA * NB * NC];
#pragma unroll 1
            for (int k = 0; k < NA * NB * NC; ++k) g[k] = 0.0;
            const int na = a.pure_ab ? 2 * LA + 1 : NA, nb = unit_b ? 1 : (a.pure_ab ? 2 * LB + 1 : NB);
            const int nc = point ? 1 : (a.pure_c ? 2 * LC + 1 : NC);
            const int fa = a.ab.foff[sa], fb = unit_b ? 0 : a.ab.foff[sb], fc = point ? 0 : a.cs.foff[sc];
#pragma unroll 1
            for (int q = 0; q < nc; ++q) {
                const double* row = a.G + (size_t)(fc + q) * a.ldg;
#pragma unroll 1
                for (int ka = 0; ka < na; ++ka) {
                    const long long m = fa + ka;
#pragma unroll 1
                    for (int kb = 0; kb < nb; ++kb) {
                        double v;
                        if (a.metric) {
                            v = row[m];
                        } else {
                            const long long n = fb + kb;
                            if (sa == sb && m < n) continue;  // diagonal shell pair: the lower triangle
                            long long col = m >= n ? m * (m + 1) / 2 + n : n * (n + 1) / 2 + m;
                            if (a.col_map) col = a.col_map[col];
                            v = col < 0 ? 0.0 : row[col];
                        }
                        g[(ka * NB + kb) * NC + q] = v;
                    }
                }
            }
            if (a.pure_c && !point) from_pure<LC, NA * NB, NC, 1, 1>(a.pure, g);
            if (a.pure_ab) {
                from_pure<LB, NA, NB * NC, NC, NC>(a.pure, g);
                from_pure<LA, 1, 0, NB * NC, NB * NC>(a.pure, g);
            }
            const double* Cc = point ? a.charge_xyz + 3 * sc : a.cs.xyz + 3 * sc;
            const int npc = point ? 1 : a.cs.nprim[sc], pc0 = point ? 0 : a.cs.poff[sc];
            constexpr double TWO_PI_52 = 34.986836655249725;
            constexpr double SGN = (LC & 1) ? -1.0 : 1.0;
#pragma unroll 1
            for (int k = 0; k < npp; ++k) {
                const double* w = shp + (size_t)k * PPW;
                const double p = w[0], ea2 = 2.0 * w[5], eb2 = 2.0 * w[6];
                const double* E[3] = {w + 7, w + 7 + ED, w + 7 + 2 * ED};
#pragma unroll 1
                for (int kc = 0; kc < npc; ++kc) {
                    // a fitting Gaussian of exponent c, or a point charge (alpha = p, 2 pi / p)
                    const double c = point ? 1.0 : a.cs.exps[pc0 + kc];
                    const double pc = p + c, alpha = point ? p : p * c / pc;
                    const double X = w[1] - Cc[0], Y = w[2] - Cc[1], Z = w[3] - Cc[2];
                    double F[L + 1];
                    boys<L>(a.boys, alpha * (X * X + Y * Y + Z * Z), F);
                    double R[NTL];
                    hermite_r<L, false>(alpha, X, Y, Z, F, R);
                    const double pref = point ? -6.283185307179586 / p * w[4] * a.charges[sc]
                                              : SGN * TWO_PI_52 / (p * c * sqrt(pc)) * w[4] * a.cs.coefs[pc0 + kc];
                    double Ec[(LC + 1) * (LC + 1)];
#pragma unroll
                    for (int q = 0; q < (LC + 1) * (LC + 1); ++q) Ec[q] = 0.0;
                    Ec[0] = 1.0;
                    const double o2c = 0.5 / c;
#pragma unroll
                    for (int i = 0; i < LC; ++i)
#pragma unroll
                        for (int t = 0; t <= LC; ++t)
                            if (t <= i + 1) {
                                double v = 0.0;
                                if (t > 0) v += o2c * Ec[i * (LC + 1) + t - 1];
                                if (t + 1 <= i) v += (t + 1) * Ec[i * (LC + 1) + t + 1];
                                Ec[(i + 1) * (LC + 1) + t] = v;
                            }
#pragma unroll 1
                    for (int kq = 0; kq < NC; ++kq) {
                        double W[NTW];
                        ket_sum_loop<LW, LC, L>(Ec, R, cart_x(LC, kq), cart_y(kq), cart_z(kq), W);
#pragma unroll 1
                        for (int ka = 0; ka < NA; ++ka)
#pragma unroll 1
                            for (int kb = 0; kb < NB; ++kb) {
                                const double gv = g[(ka * NB + kb) * NC + kq];
                                if (gv == 0.0) continue;
                                const int ii[3] = {cart_x(LA, ka), cart_y(ka), cart_z(ka)};
                                const int jj[3] = {cart_x(LB, kb), cart_y(kb), cart_z(kb)};
                                const double* e0[3];  // E(i, j) rows of the three dimensions
#pragma unroll
                                for (int d = 0; d < 3; ++d) e0[d] = E[d] + (ii[d] * (LB + 2) + jj[d]) * TE;
                                const double f = pref * gv;
#pragma unroll
                                for (int d = 0; d < 3; ++d) {
                                    // d/dA_d: 2a E(i+1, j) - i E(i-1, j) in dimension d
                                    double dA[TE], dB[TE];
                                    const double* up = E[d] + ((ii[d] + 1) * (LB + 2) + jj[d]) * TE;
                                    const double* dn = E[d] + ((ii[d] > 0 ? ii[d] - 1 : 0) * (LB + 2) + jj[d]) * TE;
                                    const double* upb = E[d] + (ii[d] * (LB + 2) + jj[d] + 1) * TE;
                                    const double* dnb = E[d] + (ii[d] * (LB + 2) + (jj[d] > 0 ? jj[d] - 1 : 0)) * TE;
#pragma unroll
                                    for (int t = 0; t < TE; ++t) {
                                        dA[t] = ea2 * up[t] - (ii[d] > 0 ? ii[d] * dn[t] : 0.0);
                                        dB[t] = eb2 * upb[t] - (jj[d] > 0 ? jj[d] * dnb[t] : 0.0);
                                    }
                                    const int n0 = ii[0] + jj[0], n1 = ii[1] + jj[1], n2 = ii[2] + jj[2];
                                    double sa_, sb_;
                                    if (d == 0) {
                                        sa_ = bra_sum_loop<LW>(dA, e0[1], e0[2], n0 + 1, n1, n2, W);
                                        sb_ = unit_b ? 0.0 : bra_sum_loop<LW>(dB, e0[1], e0[2], n0 + 1, n1, n2, W);
                                    } else if (d == 1) {
                                        sa_ = bra_sum_loop<LW>(e0[0], dA, e0[2], n0, n1 + 1, n2, W);
                                        sb_ = unit_b ? 0.0 : bra_sum_loop<LW>(e0[0], dB, e0[2], n0, n1 + 1, n2, W);
                                    } else {
                                        sa_ = bra_sum_loop<LW>(e0[0], e0[1], dA, n0, n1, n2 + 1, W);
                                        sb_ = unit_b ? 0.0 : bra_sum_loop<LW>(e0[0], e0[1], dB, n0, n1, n2 + 1, W);
                                    }
                                    gA[d] = fma(f, sa_, gA[d]);
                                    gB[d] = fma(f, sb_, gB[d]);
                                }
                            }
                    }
                }
            }
        }
    }
    // the pair's atoms are the block's: one sum per component; the fitting shells' atoms per thread
#pragma unroll
    for (int d = 0; d < 3; ++d) {
        red[d][threadIdx.x] = gA[d];
        red[3 + d][threadIdx.x] = gB[d];
    }
    __syncthreads();
    if (threadIdx.x < 6) {
        double s = 0.0;
        for (int i = 0; i < (int)blockDim.x; ++i) s += red[threadIdx.x][i];
        const int at = threadIdx.x < 3 ? atomA : atomB;
        if (s != 0.0) atomicAdd(a.grad + 3 * at + threadIdx.x % 3, s);
    }
    if (atomC >= 0) {
#pragma unroll
        for (int d = 0; d < 3; ++d) {
            const double s = gA[d] + gB[d];
            if (s != 0.0) atomicAdd(a.grad + 3 * atomC + d, -s);
        }
    }
}

using Eri3Kernel = void (*)(const Eri3Args);
int ppw(int la, int lb);

using Eri3GradKernel = void (*)(const Eri3GradArgs);
int ppw_grad(int la, int lb);

// the kernel of class (la >= lb, lc), one function per fitting-shell angular momentum lc,
// each in its own translation unit (ints3c_lc<lc>.cu) so that the classes compile in parallel
Eri3GradKernel pick_grad_lc0(int la, int lb);
Eri3GradKernel pick_grad_lc1(int la, int lb);
Eri3GradKernel pick_grad_lc2(int la, int lb);
Eri3GradKernel pick_grad_lc3(int la, int lb);
Eri3GradKernel pick_grad_lc4(int la, int lb);
Eri3Kernel pick_lc0(int la, int lb);
Eri3Kernel pick_lc1(int la, int lb);
Eri3Kernel pick_lc2(int la, int lb);
Eri3Kernel pick_lc3(int la, int lb);
Eri3Kernel pick_lc4(int la, int lb);

// the class kernels of one lc: pairs of primary shells up to f, and (fitting shell up to g,
// unit function) for the metric
template <int LC>
Eri3Kernel pick_pair(int la, int lb) {
    switch (la * 8 + lb) {
        case 0 * 8 + 0: return eri3c_kernel<0, 0, LC>;
        case 1 * 8 + 0: return eri3c_kernel<1, 0, LC>;
        case 1 * 8 + 1: return eri3c_kernel<1, 1, LC>;
        case 2 * 8 + 0: return eri3c_kernel<2, 0, LC>;
        case 2 * 8 + 1: return eri3c_kernel<2, 1, LC>;
        case 2 * 8 + 2: return eri3c_kernel<2, 2, LC>;
        case 3 * 8 + 0: return eri3c_kernel<3, 0, LC>;
        case 3 * 8 + 1: return eri3c_kernel<3, 1, LC>;
        case 3 * 8 + 2: return eri3c_kernel<3, 2, LC>;
        case 3 * 8 + 3: return eri3c_kernel<3, 3, LC>;
        case 4 * 8 + 0: return eri3c_kernel<4, 0, LC>;
        default: return nullptr;
    }
}

template <int LC>
Eri3GradKernel pick_grad_pair(int la, int lb) {
    switch (la * 8 + lb) {
        case 0 * 8 + 0: return eri3c_grad_kernel<0, 0, LC>;
        case 1 * 8 + 0: return eri3c_grad_kernel<1, 0, LC>;
        case 1 * 8 + 1: return eri3c_grad_kernel<1, 1, LC>;
        case 2 * 8 + 0: return eri3c_grad_kernel<2, 0, LC>;
        case 2 * 8 + 1: return eri3c_grad_kernel<2, 1, LC>;
        case 2 * 8 + 2: return eri3c_grad_kernel<2, 2, LC>;
        case 3 * 8 + 0: return eri3c_grad_kernel<3, 0, LC>;
        case 3 * 8 + 1: return eri3c_grad_kernel<3, 1, LC>;
        case 3 * 8 + 2: return eri3c_grad_kernel<3, 2, LC>;
        case 3 * 8 + 3: return eri3c_grad_kernel<3, 3, LC>;
        case 4 * 8 + 0: return eri3c_grad_kernel<4, 0, LC>;
        default: return nullptr;
    }
}

}  // namespace ints
}  // namespace gdfjk
