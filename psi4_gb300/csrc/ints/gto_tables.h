// gto_tables.h — tables of Cartesian Gaussians shared by the host integral provider
// (gdf_ints.cpp) and the device 3-index integrals (jk/ints3c.cu), so that both use the same
// component order, solid-harmonic coefficients, Boys grid and shell normalisation.
//
//   * Cartesian components of l in the order x^l, x^(l-1) y, x^(l-1) z, x^(l-2) y^2, ...
//   * solid harmonics from the closed form of Helgaker, Jørgensen & Olsen, "Molecular
//     Electronic-Structure Theory", eq. 6.4.47-6.4.50, rows in the order m = 0, +1, -1, +2, ...
//   * Boys function F_n(T) on a grid from the convergent series
//     F_n(T) = e^-T sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1)) in long double;
//   * primitive normalisation of the x^l component, then of the contraction.
#pragma once

#include <cmath>
#include <cstdlib>
#include <vector>

namespace gto {

inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }

inline double dfact(int n) {  // n!! with (-1)!! = 0!! = 1
    double r = 1.0;
    for (int k = n; k > 1; k -= 2) r *= k;
    return r;
}
inline double fact(int n) {
    double r = 1.0;
    for (int k = 2; k <= n; ++k) r *= k;
    return r;
}
inline double binom(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    return fact(n) / (fact(k) * fact(n - k));
}

// exponents (x, y, z) of Cartesian component k of angular momentum l
inline void cart_component(int l, int k, int* e) {
    int c = 0;
    for (int i = l; i >= 0; --i)
        for (int j = l - i; j >= 0; --j) {
            if (c == k) {
                e[0] = i;
                e[1] = j;
                e[2] = l - i - j;
                return;
            }
            ++c;
        }
}

// Cartesian -> real solid harmonic matrix, (2l+1) x ncart(l), row-major.
inline std::vector<double> pure_matrix(int l) {
    const int nc = ncart(l);
    std::vector<double> c((size_t)(2 * l + 1) * nc, 0.0);
    std::vector<int> comp((size_t)3 * nc);
    for (int k = 0; k < nc; ++k) cart_component(l, k, &comp[3 * k]);
    for (int r = 0; r < 2 * l + 1; ++r) {
        const int m = (r == 0) ? 0 : ((r % 2 == 1) ? (r + 1) / 2 : -(r / 2));
        const int am = std::abs(m);
        double* row = &c[(size_t)r * nc];
        const int vstart2 = (m >= 0) ? 0 : 1;  // 2 v_m
        for (int t = 0; t <= (l - am) / 2; ++t)
            for (int u = 0; u <= t; ++u)
                for (int v2 = vstart2; v2 <= am; v2 += 2) {
                    const double sgn = (((t + (v2 - vstart2) / 2) % 2) == 0) ? 1.0 : -1.0;
                    const double coef =
                        sgn * std::pow(0.25, t) * binom(l, t) * binom(l - t, am + t) * binom(t, u) * binom(am, v2);
                    const int px = 2 * t + am - 2 * u - v2, py = 2 * u + v2, pz = l - 2 * t - am;
                    for (int k = 0; k < nc; ++k)
                        if (comp[3 * k] == px && comp[3 * k + 1] == py && comp[3 * k + 2] == pz) row[k] += coef;
                }
        // normalise: the components share the radial part and the x^l normalisation
        double nrm = 0.0;
        for (int a = 0; a < nc; ++a)
            for (int b = 0; b < nc; ++b) {
                const int sx = comp[3 * a] + comp[3 * b], sy = comp[3 * a + 1] + comp[3 * b + 1],
                          sz = comp[3 * a + 2] + comp[3 * b + 2];
                if ((sx | sy | sz) & 1) continue;
                nrm += row[a] * row[b] * dfact(sx - 1) * dfact(sy - 1) * dfact(sz - 1) / dfact(2 * l - 1);
            }
        const double s = 1.0 / std::sqrt(nrm);
        for (int k = 0; k < nc; ++k) row[k] *= s;
    }
    return c;
}

// Boys grid: tab[g * stride + n] = F_n(g h), g < ngrid, n < stride.
inline std::vector<double> boys_grid(int ngrid, int stride, double h) {
    std::vector<double> tab((size_t)ngrid * stride, 0.0);
    for (int g = 0; g < ngrid; ++g) {
        const long double T = static_cast<long double>(g) * h;
        for (int n = 0; n < stride; ++n) {
            long double term = 1.0L / (2 * n + 1);
            long double sum = term;
            for (int k = 1; k < 2000; ++k) {
                term *= 2.0L * T / (2 * n + 2 * k + 1);
                sum += term;
                if (term < 1e-22L * sum) break;
            }
            tab[(size_t)g * stride + n] = static_cast<double>(std::exp(-T) * sum);
        }
    }
    return tab;
}
// grid of the Boys tables: F_n(T) by a KT-term Taylor expansion about the nearest grid point
// for T < TMAX, the asymptotic form above
constexpr double BOYS_TMAX = 40.0;
constexpr double BOYS_H = 0.025;
constexpr int BOYS_KT = 7;
inline int boys_ngrid() { return static_cast<int>(BOYS_TMAX / BOYS_H) + 2; }

// contraction coefficients c[0..nprim) of a shell, normalised in place: each primitive's x^l
// component, then the contracted function
inline void normalise_shell(int l, int nprim, const double* a, double* c) {
    for (int k = 0; k < nprim; ++k)
        c[k] *= std::pow(2.0 * a[k] / M_PI, 0.75) * std::pow(4.0 * a[k], 0.5 * l) / std::sqrt(dfact(2 * l - 1));
    double nrm = 0.0;
    for (int i = 0; i < nprim; ++i)
        for (int j = 0; j < nprim; ++j) {
            const double g = a[i] + a[j];
            nrm += c[i] * c[j] * std::pow(M_PI / g, 1.5) * dfact(2 * l - 1) / std::pow(2.0 * g, l);
        }
    const double sc = 1.0 / std::sqrt(nrm);
    for (int k = 0; k < nprim; ++k) c[k] *= sc;
}

}  // namespace gto
