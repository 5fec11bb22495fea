// gdf_ints.cpp — host Gaussian integral provider (McMurchie–Davidson) for the DF-JK engine.
//
// Supplies, on the host, the integrals psi4 takes from libint2 for the density-fitted
// Fock build: the Coulomb metric (P|Q) (fittingmetric.cc:72), the 3-index (P|mn)
// (dfhelper.cc:1284-1347), the Schwarz diagonal (mn|mn) (dfhelper.cc:336-366), the
// one-electron S, T, V the SCF needs, and their first derivatives for the nuclear
// gradient (jk_grad.cc:834-1245, scf_grad.cc:196-220).
//
// Method (Helgaker, Jørgensen & Olsen, "Molecular Electronic-Structure Theory", ch. 9):
//   * Gaussian product -> Hermite expansion coefficients E^{ij}_t by the two-term
//     recurrences (9.5.6-9.5.7);
//   * Coulomb-type integrals from the Hermite integrals R^n_{tuv} (9.9.18-9.9.20)
//     seeded by the Boys function F_n(T);
//   * first derivatives by differentiating the Cartesian Gaussians,
//     d/dA_x x_A^i e^{-a x_A^2} = 2a x_A^{i+1} e^{..} - i x_A^{i-1} e^{..}, folded into
//     derivative Hermite coefficients, with translational invariance for the last centre.
// Boys function: a grid of F_n(T) built from the convergent series
//   F_n(T) = e^{-T} sum_k (2T)^k / ((2n+1)(2n+3)...(2n+2k+1))
// evaluated by a 7-term Taylor expansion around the nearest grid point (dF_n/dT = -F_{n+1})
// plus downward recursion; for large T the asymptotic F_0 = sqrt(pi/T)/2 and upward
// recursion.  Solid harmonics from the closed form in MEST eq. 6.4.47-6.4.50.

#include "gdfints.h"
#include "gto_tables.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

thread_local std::string g_err;

int fail(const std::string& msg, int code = -1) {
    g_err = msg;
    return code;
}

constexpr int MAXL = 5;                  // highest shell angular momentum supported (h)
constexpr int EDIM = MAXL + 3;           // i, j range in Hermite tables (l + 2 for kinetic)
constexpr int TDIM = 2 * MAXL + 6;       // t range in Hermite tables
constexpr int RDIM = 4 * MAXL + 4;       // R cube edge (total Hermite order + 1)

inline int ncart(int l) { return (l + 1) * (l + 2) / 2; }
inline int ntuv(int L) { return (L + 1) * (L + 2) * (L + 3) / 6; }

double dfact(int n) {  // n!! with (-1)!! = 0!! = 1
    double r = 1.0;
    for (int k = n; k > 1; k -= 2) r *= k;
    return r;
}
double fact(int n) {
    double r = 1.0;
    for (int k = 2; k <= n; ++k) r *= k;
    return r;
}
double binom(int n, int k) {
    if (k < 0 || k > n) return 0.0;
    return fact(n) / (fact(k) * fact(n - k));
}

// Cartesian components of angular momentum l in standard order.
struct CartTable {
    int comp[MAXL + 3][64][3];
    CartTable() {
        for (int l = 0; l <= MAXL + 2; ++l) {
            int c = 0;
            for (int i = l; i >= 0; --i)
                for (int j = l - i; j >= 0; --j) {
                    comp[l][c][0] = i;
                    comp[l][c][1] = j;
                    comp[l][c][2] = l - i - j;
                    ++c;
                }
        }
    }
};
const CartTable& carts() {
    static CartTable t;
    return t;
}

// Hermite index positions for t+u+v <= L, ordered by (t, u, v) lexicographically.
struct TuvTable {
    std::vector<int> t_of[RDIM], u_of[RDIM], v_of[RDIM];  // per L, list of tuv
    TuvTable() {
        for (int L = 0; L < RDIM; ++L) {
            for (int t = 0; t <= L; ++t)
                for (int u = 0; u <= L - t; ++u)
                    for (int v = 0; v <= L - t - u; ++v) {
                        t_of[L].push_back(t);
                        u_of[L].push_back(u);
                        v_of[L].push_back(v);
                    }
        }
    }
};
const TuvTable& tuvs() {
    static TuvTable t;
    return t;
}

// ---------------------------------------------------------------- Boys function
struct Boys {
    static constexpr int NMAX = RDIM + 2;
    static constexpr int KT = gto::BOYS_KT;
    static constexpr double TMAX = gto::BOYS_TMAX;
    static constexpr double H = gto::BOYS_H;
    int ngrid;
    int stride;
    std::vector<double> tab;
    Boys() {
        ngrid = gto::boys_ngrid();
        stride = NMAX + KT + 1;
        tab = gto::boys_grid(ngrid, stride, H);
    }
    // F[0..n]
    void eval(int n, double T, double* F) const {
        if (T < TMAX) {
            int g = static_cast<int>(T / H + 0.5);
            double dT = g * H - T;  // F_n(T) = sum_k F_{n+k}(T_g) (T_g - T)^k / k!
            const double* row = &tab[static_cast<size_t>(g) * stride];
            double f = 0.0, pw = 1.0;
            for (int k = 0; k < KT; ++k) {
                f += row[n + k] * pw;
                pw *= dT / (k + 1);
            }
            F[n] = f;
            if (n > 0) {
                double e = std::exp(-T);
                for (int m = n - 1; m >= 0; --m) F[m] = (2.0 * T * F[m + 1] + e) / (2 * m + 1);
            }
        } else {
            double e = std::exp(-T);
            F[0] = 0.5 * std::sqrt(M_PI / T) * std::erf(std::sqrt(T));
            for (int m = 0; m < n; ++m) F[m + 1] = ((2 * m + 1) * F[m] - e) / (2.0 * T);
        }
    }
};
const Boys& boys() {
    static Boys b;
    return b;
}

// ---------------------------------------------------------------- solid harmonics
// cart -> pure coefficient matrix (2l+1) x ncart(l), rows in Gaussian order m = 0, +1, -1, ...
struct PureTable {
    std::vector<double> c[MAXL + 1];
    PureTable() {
        for (int l = 0; l <= MAXL; ++l) c[l] = gto::pure_matrix(l);
    }
};
const PureTable& pures() {
    static PureTable p;
    return p;
}

}  // namespace

// ---------------------------------------------------------------- basis
struct gdfints_basis_s {
    struct Shell {
        int l, nprim, nfunc, ncart, off, atom;
        double O[3];
        std::vector<double> a, c;  // exponents, normalised coefficients (x^l norm included)
    };
    std::vector<Shell> sh;
    int puream = 1;
    int nbf = 0;
};

namespace {

using Basis = gdfints_basis_s;
using Shell = gdfints_basis_s::Shell;

Shell unit_shell(const double* O) {
    Shell s;
    s.l = 0;
    s.nprim = 1;
    s.nfunc = 1;
    s.ncart = 1;
    s.off = 0;
    s.atom = -1;
    s.O[0] = O[0];
    s.O[1] = O[1];
    s.O[2] = O[2];
    s.a = {0.0};
    s.c = {1.0};
    return s;
}

// 1D Hermite coefficients E[i][j][t] for a primitive pair, i <= imax, j <= jmax.
// E[0][0][0] = exp(-mu X_AB^2).
struct Herm1D {
    double e[EDIM][EDIM][TDIM];
};
void hermite_1d(int imax, int jmax, double a, double b, double A, double B, Herm1D& H) {
    double p = a + b;
    double mu = a * b / p;
    double P = (a * A + b * B) / p;
    double XPA = P - A, XPB = P - B, XAB = A - B;
    double oo2p = 0.5 / p;
    for (int i = 0; i <= imax; ++i)
        for (int j = 0; j <= jmax; ++j)
            for (int t = 0; t <= i + j + 1 && t < TDIM; ++t) H.e[i][j][t] = 0.0;
    H.e[0][0][0] = std::exp(-mu * XAB * XAB);
    for (int i = 0; i < imax; ++i) {
        for (int t = 0; t <= i + 1; ++t) {
            double v = XPA * H.e[i][0][t];
            if (t > 0) v += oo2p * H.e[i][0][t - 1];
            if (t + 1 <= i) v += (t + 1) * H.e[i][0][t + 1];
            H.e[i + 1][0][t] = v;
        }
    }
    for (int i = 0; i <= imax; ++i)
        for (int j = 0; j < jmax; ++j)
            for (int t = 0; t <= i + j + 1; ++t) {
                double v = XPB * H.e[i][j][t];
                if (t > 0) v += oo2p * H.e[i][j][t - 1];
                if (t + 1 <= i + j) v += (t + 1) * H.e[i][j][t + 1];
                H.e[i][j + 1][t] = v;
            }
}

// R^0_{tuv} for t+u+v <= L into cube R[(t*RDIM+u)*RDIM+v]
void hermite_R(int L, double alpha, double X, double Y, double Z, double* R, double* W) {
    double F[RDIM + 4];
    double T = alpha * (X * X + Y * Y + Z * Z);
    boys().eval(L, T, F);
    auto I = [](int t, int u, int v) { return (t * RDIM + u) * RDIM + v; };
    double* cur = R;
    double* prev = W;
    // Start at n = L and go down; buffers alternate so that n = 0 ends in R.
    if (L % 2 == 1) std::swap(cur, prev);
    double m2a = -2.0 * alpha;
    for (int n = L; n >= 0; --n) {
        int Lr = L - n;
        cur[I(0, 0, 0)] = std::pow(m2a, n) * F[n];
        for (int t = 0; t <= Lr; ++t)
            for (int u = 0; u <= Lr - t; ++u)
                for (int v = 0; v <= Lr - t - u; ++v) {
                    if (t + u + v == 0) continue;
                    double val;
                    if (t > 0) {
                        val = X * prev[I(t - 1, u, v)];
                        if (t > 1) val += (t - 1) * prev[I(t - 2, u, v)];
                    } else if (u > 0) {
                        val = Y * prev[I(t, u - 1, v)];
                        if (u > 1) val += (u - 1) * prev[I(t, u - 2, v)];
                    } else {
                        val = Z * prev[I(t, u, v - 1)];
                        if (v > 1) val += (v - 1) * prev[I(t, u, v - 2)];
                    }
                    cur[I(t, u, v)] = val;
                }
        std::swap(cur, prev);
    }
}

// Hermite matrix of a primitive pair: H[ab][k] over the tuv list of order Lh.
// sel: 0 = plain; 1..3 = d/dA_{x,y,z}; 4..6 = d/dB_{x,y,z}.
void hermite_matrix(int la, int lb, double a, double b, const Herm1D* E /*x,y,z*/, int sel, int Lh, double* H) {
    const auto& ct = carts();
    const auto& tv = tuvs();
    int na = ncart(la), nb = ncart(lb), nt = ntuv(Lh);
    const auto& T = tv.t_of[Lh];
    const auto& U = tv.u_of[Lh];
    const auto& V = tv.v_of[Lh];
    int dir = (sel == 0) ? -1 : (sel - 1) % 3;
    bool onA = sel >= 1 && sel <= 3;
    for (int ia = 0; ia < na; ++ia) {
        const int* ca = ct.comp[la][ia];
        for (int ib = 0; ib < nb; ++ib) {
            const int* cb = ct.comp[lb][ib];
            double* row = H + static_cast<size_t>(ia * nb + ib) * nt;
            for (int k = 0; k < nt; ++k) {
                int tt[3] = {T[k], U[k], V[k]};
                double prod = 1.0;
                for (int d = 0; d < 3; ++d) {
                    int i = ca[d], j = cb[d], t = tt[d];
                    double val;
                    if (d != dir) {
                        val = (t <= i + j) ? E[d].e[i][j][t] : 0.0;
                    } else if (onA) {
                        val = (t <= i + j + 1) ? 2.0 * a * E[d].e[i + 1][j][t] : 0.0;
                        if (i > 0 && t <= i + j - 1) val -= i * E[d].e[i - 1][j][t];
                    } else {
                        val = (t <= i + j + 1) ? 2.0 * b * E[d].e[i][j + 1][t] : 0.0;
                        if (j > 0 && t <= i + j - 1) val -= j * E[d].e[i][j - 1][t];
                    }
                    prod *= val;
                    if (prod == 0.0) break;
                }
                row[k] = prod;
            }
        }
    }
}

// Cartesian -> pure transform of index `which` of a block with dims n[0..3].
void to_pure(const int* l, const int* pure_flags, int ndim, std::vector<double>& blk, std::vector<double>& tmp) {
    const auto& pt = pures();
    int dims[4];
    for (int d = 0; d < ndim; ++d) dims[d] = ncart(l[d]);
    for (int d = 0; d < ndim; ++d) {
        // s needs no transform; pure p comes out in the order (z, x, y) = m (0, +1, -1)
        if (!pure_flags[d] || l[d] == 0) continue;
        int nc = dims[d], np = 2 * l[d] + 1;
        size_t outer = 1, inner = 1;
        for (int e = 0; e < d; ++e) outer *= dims[e];
        for (int e = d + 1; e < ndim; ++e) inner *= dims[e];
        tmp.assign(outer * np * inner, 0.0);
        const double* C = pt.c[l[d]].data();
        for (size_t o = 0; o < outer; ++o)
            for (int r = 0; r < np; ++r) {
                double* dst = &tmp[(o * np + r) * inner];
                for (int k = 0; k < nc; ++k) {
                    double cf = C[r * nc + k];
                    if (cf == 0.0) continue;
                    const double* src = &blk[(o * nc + k) * inner];
                    for (size_t i = 0; i < inner; ++i) dst[i] += cf * src[i];
                }
            }
        dims[d] = np;
        blk.swap(tmp);
    }
}

struct Scratch {
    std::vector<double> R, W, Rm, Hb, Hk, Tm, blk, tmp;
    std::vector<double> Hbd[7], Hkd[4], Tmd[4];
};

// Contracted Cartesian (AB|CD) (bra pair AB, ket pair CD; B/D may be unit shells).
// out[ab*ncd + cd].  When deriv != 0 also fills dout[9][ab*ncd+cd]: derivatives with respect
// to A_xyz (0-2), B_xyz (3-5), C_xyz (6-8); the D centre follows by translation invariance.
// omega > 0: the long-range operator erf(omega r)/r instead of 1/r (psi4's erf_eri, used for
// wK): the reduced exponent alpha of each primitive quartet becomes
// alpha_w = alpha omega^2 / (alpha + omega^2) in the Boys argument and the Hermite recursion,
// and the prefactor gains sqrt(alpha_w / alpha)  (erf(wr)/r = 2/sqrt(pi) int_0^w exp(-t^2 r^2) dt).
void eri_cart(const Shell& A, const Shell& B, const Shell& C, const Shell& D, Scratch& s, double* out, int deriv,
              double* dout, double omega = 0.0) {
    int la = A.l, lb = B.l, lc = C.l, ld = D.l;
    int nab = ncart(la) * ncart(lb), ncd = ncart(lc) * ncart(ld);
    int Lb = la + lb + deriv, Lk = lc + ld + deriv;
    int L = Lb + Lk;
    int ntb = ntuv(Lb), ntk = ntuv(Lk);
    const auto& tv = tuvs();
    s.R.resize(RDIM * RDIM * RDIM);
    s.W.resize(RDIM * RDIM * RDIM);
    s.Rm.resize(static_cast<size_t>(ntb) * ntk);
    s.Hb.resize(static_cast<size_t>(nab) * ntb);
    s.Hk.resize(static_cast<size_t>(ncd) * ntk);
    s.Tm.resize(static_cast<size_t>(ntb) * ncd);
    std::fill(out, out + static_cast<size_t>(nab) * ncd, 0.0);
    if (deriv) {
        for (int k = 0; k < 7; ++k) s.Hbd[k].resize(static_cast<size_t>(nab) * ntb);
        for (int k = 0; k < 4; ++k) {
            s.Hkd[k].resize(static_cast<size_t>(ncd) * ntk);
            s.Tmd[k].resize(static_cast<size_t>(ntb) * ncd);
        }
        std::fill(dout, dout + 9 * static_cast<size_t>(nab) * ncd, 0.0);
    }
    const auto& Tb = tv.t_of[Lb];
    const auto& Ub = tv.u_of[Lb];
    const auto& Vb = tv.v_of[Lb];
    const auto& Tk = tv.t_of[Lk];
    const auto& Uk = tv.u_of[Lk];
    const auto& Vk = tv.v_of[Lk];
    const double pi52 = 2.0 * std::pow(M_PI, 2.5);
    Herm1D Eab[3], Ecd[3];
    for (int pa = 0; pa < A.nprim; ++pa)
        for (int pb = 0; pb < B.nprim; ++pb) {
            double a = A.a[pa], b = B.a[pb];
            double p = a + b;
            double P[3];
            for (int d = 0; d < 3; ++d) {
                P[d] = (a * A.O[d] + b * B.O[d]) / p;
                hermite_1d(la + 1 + (deriv ? 1 : 0), lb + (deriv ? 1 : 0), a, b, A.O[d], B.O[d], Eab[d]);
            }
            double cab = A.c[pa] * B.c[pb];
            hermite_matrix(la, lb, a, b, Eab, 0, Lb, s.Hb.data());
            if (deriv)
                for (int k = 1; k < 7; ++k) hermite_matrix(la, lb, a, b, Eab, k, Lb, s.Hbd[k].data());
            for (int pc = 0; pc < C.nprim; ++pc)
                for (int pd = 0; pd < D.nprim; ++pd) {
                    double c = C.a[pc], dd = D.a[pd];
                    double q = c + dd;
                    double Q[3];
                    for (int d = 0; d < 3; ++d) {
                        Q[d] = (c * C.O[d] + dd * D.O[d]) / q;
                        hermite_1d(lc + 1 + (deriv ? 1 : 0), ld + (deriv ? 1 : 0), c, dd, C.O[d], D.O[d], Ecd[d]);
                    }
                    double pref = pi52 / (p * q * std::sqrt(p + q)) * cab * C.c[pc] * D.c[pd];
                    double alpha = p * q / (p + q);
                    if (omega > 0.0) {
                        const double aw = alpha * omega * omega / (alpha + omega * omega);
                        pref *= std::sqrt(aw / alpha);
                        alpha = aw;
                    }
                    hermite_R(L, alpha, P[0] - Q[0], P[1] - Q[1], P[2] - Q[2], s.R.data(), s.W.data());
                    // ket Hermite matrix with (-1)^{tau+nu+phi}
                    hermite_matrix(lc, ld, c, dd, Ecd, 0, Lk, s.Hk.data());
                    if (deriv)
                        for (int k = 1; k < 4; ++k) hermite_matrix(lc, ld, c, dd, Ecd, k, Lk, s.Hkd[k].data());
                    for (int i = 0; i < ntb; ++i)
                        for (int j = 0; j < ntk; ++j) {
                            int t = Tb[i] + Tk[j], u = Ub[i] + Uk[j], v = Vb[i] + Vk[j];
                            double sg = ((Tk[j] + Uk[j] + Vk[j]) & 1) ? -1.0 : 1.0;
                            s.Rm[static_cast<size_t>(i) * ntk + j] = sg * s.R[(t * RDIM + u) * RDIM + v];
                        }
                    // Tm[i][cd] = sum_j Rm[i][j] Hk[cd][j]
                    auto contract_ket = [&](const std::vector<double>& Hk, std::vector<double>& Tm) {
                        for (int i = 0; i < ntb; ++i) {
                            const double* rr = &s.Rm[static_cast<size_t>(i) * ntk];
                            double* tr = &Tm[static_cast<size_t>(i) * ncd];
                            for (int cd = 0; cd < ncd; ++cd) {
                                const double* hk = &Hk[static_cast<size_t>(cd) * ntk];
                                double acc = 0.0;
                                for (int j = 0; j < ntk; ++j) acc += rr[j] * hk[j];
                                tr[cd] = acc;
                            }
                        }
                    };
                    auto contract_bra = [&](const std::vector<double>& Hb, const std::vector<double>& Tm, double* o) {
                        for (int ab = 0; ab < nab; ++ab) {
                            const double* hb = &Hb[static_cast<size_t>(ab) * ntb];
                            double* orow = o + static_cast<size_t>(ab) * ncd;
                            for (int i = 0; i < ntb; ++i) {
                                double h = hb[i];
                                if (h == 0.0) continue;
                                h *= pref;
                                const double* tr = &Tm[static_cast<size_t>(i) * ncd];
                                for (int cd = 0; cd < ncd; ++cd) orow[cd] += h * tr[cd];
                            }
                        }
                    };
                    contract_ket(s.Hk, s.Tm);
                    contract_bra(s.Hb, s.Tm, out);
                    if (deriv) {
                        size_t blk = static_cast<size_t>(nab) * ncd;
                        for (int k = 1; k < 7; ++k) contract_bra(s.Hbd[k], s.Tm, dout + (k - 1) * blk);
                        for (int k = 1; k < 4; ++k) {
                            contract_ket(s.Hkd[k], s.Tmd[k]);
                            contract_bra(s.Hb, s.Tmd[k], dout + (5 + k) * blk);
                        }
                    }
                }
        }
}

int nthreads() {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
int thread_id() {
#ifdef _OPENMP
    return omp_get_thread_num();
#else
    return 0;
#endif
}

// Transform a Cartesian block (dims = ncart of ls) to pure/cartesian functions of the basis.
void finish_block(const int* ls, const int* pureflags, int nd, std::vector<double>& blk, std::vector<double>& tmp) {
    to_pure(ls, pureflags, nd, blk, tmp);
}

}  // namespace

extern "C" {

const char* gdfints_last_error(void) { return g_err.c_str(); }

int gdfints_boys(int n, double T, double* F) {
    if (n < 0 || n > Boys::NMAX) return fail("boys: order out of range");
    boys().eval(n, T, F);
    return 0;
}

int gdfints_basis_create(int nshell, const int* l, const int* nprim, const int* prim_offset, const double* exps,
                         const double* coefs, const double* xyz, const int* atom, int puream, gdfints_basis_t* out) {
    try {
        auto* b = new gdfints_basis_s();
        b->puream = puream ? 1 : 0;
        int off = 0;
        for (int s = 0; s < nshell; ++s) {
            Shell sh;
            sh.l = l[s];
            if (sh.l < 0 || sh.l > MAXL) {
                delete b;
                return fail("basis: angular momentum above the supported maximum (h)");
            }
            sh.nprim = nprim[s];
            sh.ncart = ncart(sh.l);
            sh.nfunc = b->puream ? 2 * sh.l + 1 : sh.ncart;
            sh.off = off;
            sh.atom = atom ? atom[s] : -1;
            off += sh.nfunc;
            for (int d = 0; d < 3; ++d) sh.O[d] = xyz[3 * s + d];
            sh.a.assign(exps + prim_offset[s], exps + prim_offset[s] + sh.nprim);
            sh.c.assign(coefs + prim_offset[s], coefs + prim_offset[s] + sh.nprim);
            gto::normalise_shell(sh.l, sh.nprim, sh.a.data(), sh.c.data());
            b->sh.push_back(std::move(sh));
        }
        b->nbf = off;
        // force table construction on this thread
        (void)boys();
        (void)pures();
        (void)tuvs();
        (void)carts();
        *out = b;
        return 0;
    } catch (const std::exception& e) {
        return fail(std::string("basis: ") + e.what());
    }
}

void gdfints_basis_destroy(gdfints_basis_t b) { delete b; }
int gdfints_basis_nbf(gdfints_basis_t b) { return b ? b->nbf : -1; }
int gdfints_basis_shell_offsets(gdfints_basis_t b, int* offsets) {
    for (size_t s = 0; s < b->sh.size(); ++s) offsets[s] = b->sh[s].off;
    return 0;
}

}  // extern "C"

namespace {

// ---- one-electron pieces ------------------------------------------------------
// For a primitive pair, the 1D overlap S_d(i,j) = E_d[i][j][0] sqrt(pi/p) and kinetic
// T_d(i,j) = -2 b^2 S(i,j+2) + b(2j+1) S(i,j) - j(j-1)/2 S(i,j-2).
enum OneKind { ONE_S, ONE_T };

void one_e_block(const Shell& A, const Shell& B, OneKind kind, int deriv, std::vector<double>& out,
                 std::vector<double>& dA) {
    const auto& ct = carts();
    int na = ncart(A.l), nb = ncart(B.l);
    out.assign(static_cast<size_t>(na) * nb, 0.0);
    if (deriv) dA.assign(3 * static_cast<size_t>(na) * nb, 0.0);
    Herm1D E[3];
    for (int pa = 0; pa < A.nprim; ++pa)
        for (int pb = 0; pb < B.nprim; ++pb) {
            double a = A.a[pa], b = B.a[pb], p = a + b;
            double sq = std::sqrt(M_PI / p);
            for (int d = 0; d < 3; ++d) hermite_1d(A.l + 2, B.l + 2, a, b, A.O[d], B.O[d], E[d]);
            double cc = A.c[pa] * B.c[pb];
            auto S1 = [&](int d, int i, int j) -> double {
                if (i < 0 || j < 0) return 0.0;
                return E[d].e[i][j][0] * sq;
            };
            auto T1 = [&](int d, int i, int j) -> double {
                if (i < 0 || j < 0) return 0.0;
                double v = -2.0 * b * b * S1(d, i, j + 2) + b * (2 * j + 1) * S1(d, i, j);
                if (j >= 2) v -= 0.5 * j * (j - 1) * S1(d, i, j - 2);
                return v;
            };
            for (int ia = 0; ia < na; ++ia) {
                const int* ca = ct.comp[A.l][ia];
                for (int ib = 0; ib < nb; ++ib) {
                    const int* cb = ct.comp[B.l][ib];
                    double s[3], t[3], ds[3], dt[3];
                    for (int d = 0; d < 3; ++d) {
                        int i = ca[d], j = cb[d];
                        s[d] = S1(d, i, j);
                        t[d] = T1(d, i, j);
                        if (deriv) {
                            ds[d] = 2.0 * a * S1(d, i + 1, j) - (i > 0 ? i * S1(d, i - 1, j) : 0.0);
                            dt[d] = 2.0 * a * T1(d, i + 1, j) - (i > 0 ? i * T1(d, i - 1, j) : 0.0);
                        }
                    }
                    size_t k = static_cast<size_t>(ia) * nb + ib;
                    if (kind == ONE_S) {
                        out[k] += cc * s[0] * s[1] * s[2];
                        if (deriv) {
                            dA[0 * na * nb + k] += cc * ds[0] * s[1] * s[2];
                            dA[1 * na * nb + k] += cc * s[0] * ds[1] * s[2];
                            dA[2 * na * nb + k] += cc * s[0] * s[1] * ds[2];
                        }
                    } else {
                        out[k] += cc * (t[0] * s[1] * s[2] + s[0] * t[1] * s[2] + s[0] * s[1] * t[2]);
                        if (deriv) {
                            dA[0 * na * nb + k] += cc * (dt[0] * s[1] * s[2] + ds[0] * t[1] * s[2] + ds[0] * s[1] * t[2]);
                            dA[1 * na * nb + k] += cc * (t[0] * ds[1] * s[2] + s[0] * dt[1] * s[2] + s[0] * ds[1] * t[2]);
                            dA[2 * na * nb + k] += cc * (t[0] * s[1] * ds[2] + s[0] * t[1] * ds[2] + s[0] * s[1] * dt[2]);
                        }
                    }
                }
            }
        }
}

// Nuclear attraction block and (optionally) its derivatives w.r.t. A (0-2) and B (3-5);
// the operator-centre derivative follows from translation invariance per nucleus, so it
// is returned separately per nucleus in dC (3*natom blocks) when requested.
void potential_block(const Shell& A, const Shell& B, int natom, const double* Z, const double* xyz, int deriv,
                     Scratch& s, std::vector<double>& out, std::vector<double>& dAB, std::vector<double>& dC) {
    int la = A.l, lb = B.l;
    int nab = ncart(la) * ncart(lb);
    int Lh = la + lb + deriv;
    int nt = ntuv(Lh);
    const auto& tv = tuvs();
    const auto& T = tv.t_of[Lh];
    const auto& U = tv.u_of[Lh];
    const auto& V = tv.v_of[Lh];
    out.assign(nab, 0.0);
    if (deriv) {
        dAB.assign(6 * static_cast<size_t>(nab), 0.0);
        dC.assign(3 * static_cast<size_t>(natom) * nab, 0.0);
        for (int k = 0; k < 7; ++k) s.Hbd[k].resize(static_cast<size_t>(nab) * nt);
    }
    s.Hb.resize(static_cast<size_t>(nab) * nt);
    s.R.resize(RDIM * RDIM * RDIM);
    s.W.resize(RDIM * RDIM * RDIM);
    Herm1D E[3];
    for (int pa = 0; pa < A.nprim; ++pa)
        for (int pb = 0; pb < B.nprim; ++pb) {
            double a = A.a[pa], b = B.a[pb], p = a + b;
            double P[3];
            for (int d = 0; d < 3; ++d) {
                P[d] = (a * A.O[d] + b * B.O[d]) / p;
                hermite_1d(la + 1 + deriv, lb + deriv, a, b, A.O[d], B.O[d], E[d]);
            }
            double cc = A.c[pa] * B.c[pb] * 2.0 * M_PI / p;
            hermite_matrix(la, lb, a, b, E, 0, Lh, s.Hb.data());
            if (deriv)
                for (int k = 1; k < 7; ++k) hermite_matrix(la, lb, a, b, E, k, Lh, s.Hbd[k].data());
            for (int C = 0; C < natom; ++C) {
                double X = P[0] - xyz[3 * C], Y = P[1] - xyz[3 * C + 1], Zc = P[2] - xyz[3 * C + 2];
                hermite_R(Lh + (deriv ? 1 : 0), p, X, Y, Zc, s.R.data(), s.W.data());
                double f = -Z[C] * cc;
                auto Rv = [&](int t, int u, int v) { return s.R[(t * RDIM + u) * RDIM + v]; };
                for (int ab = 0; ab < nab; ++ab) {
                    const double* h = &s.Hb[static_cast<size_t>(ab) * nt];
                    double acc = 0.0, gx = 0.0, gy = 0.0, gz = 0.0;
                    for (int k = 0; k < nt; ++k) {
                        if (h[k] == 0.0) continue;
                        acc += h[k] * Rv(T[k], U[k], V[k]);
                        if (deriv) {
                            // d/dC of R_{tuv}(P - C) = -R_{t+1,u,v} etc.
                            gx -= h[k] * Rv(T[k] + 1, U[k], V[k]);
                            gy -= h[k] * Rv(T[k], U[k] + 1, V[k]);
                            gz -= h[k] * Rv(T[k], U[k], V[k] + 1);
                        }
                    }
                    out[ab] += f * acc;
                    if (deriv) {
                        dC[(3 * C + 0) * nab + ab] += f * gx;
                        dC[(3 * C + 1) * nab + ab] += f * gy;
                        dC[(3 * C + 2) * nab + ab] += f * gz;
                        for (int kk = 1; kk < 7; ++kk) {
                            const double* hd = &s.Hbd[kk][static_cast<size_t>(ab) * nt];
                            double ad = 0.0;
                            for (int k = 0; k < nt; ++k)
                                if (hd[k] != 0.0) ad += hd[k] * Rv(T[k], U[k], V[k]);
                            dAB[(kk - 1) * nab + ab] += f * ad;
                        }
                    }
                }
            }
        }
}

// Apply the pure transform to a 2-index Cartesian block (na_c x nb_c).
void pure2(const Basis& bs, const Shell& A, const Shell& B, std::vector<double>& blk, std::vector<double>& tmp) {
    int ls[2] = {A.l, B.l};
    int pf[2] = {bs.puream, bs.puream};
    finish_block(ls, pf, 2, blk, tmp);
}

template <class F>
int one_e_driver(const Basis& b, double* M, F&& blockfn) {
    int ns = static_cast<int>(b.sh.size());
    int nbf = b.nbf;
    std::vector<std::pair<int, int>> pairs;
    for (int i = 0; i < ns; ++i)
        for (int j = 0; j <= i; ++j) pairs.emplace_back(i, j);
#pragma omp parallel
    {
        std::vector<double> blk, tmp, dA;
        Scratch s;
#pragma omp for schedule(dynamic)
        for (size_t k = 0; k < pairs.size(); ++k) {
            const Shell& A = b.sh[pairs[k].first];
            const Shell& B = b.sh[pairs[k].second];
            blockfn(A, B, s, blk, dA);
            pure2(b, A, B, blk, tmp);
            for (int i = 0; i < A.nfunc; ++i)
                for (int j = 0; j < B.nfunc; ++j) {
                    double v = blk[i * B.nfunc + j];
                    M[static_cast<size_t>(A.off + i) * nbf + B.off + j] = v;
                    M[static_cast<size_t>(B.off + j) * nbf + A.off + i] = v;
                }
        }
    }
    return 0;
}

}  // namespace

extern "C" {

int gdfints_overlap(gdfints_basis_t b, double* S) {
    return one_e_driver(*b, S, [](const Shell& A, const Shell& B, Scratch&, std::vector<double>& blk,
                                  std::vector<double>& dA) { one_e_block(A, B, ONE_S, 0, blk, dA); });
}
int gdfints_kinetic(gdfints_basis_t b, double* T) {
    return one_e_driver(*b, T, [](const Shell& A, const Shell& B, Scratch&, std::vector<double>& blk,
                                  std::vector<double>& dA) { one_e_block(A, B, ONE_T, 0, blk, dA); });
}
int gdfints_potential(gdfints_basis_t b, int natom, const double* Z, const double* xyz, double* V) {
    return one_e_driver(*b, V, [&](const Shell& A, const Shell& B, Scratch& s, std::vector<double>& blk,
                                   std::vector<double>&) {
        std::vector<double> d1, d2;
        potential_block(A, B, natom, Z, xyz, 0, s, blk, d1, d2);
    });
}

int gdfints_metric(gdfints_basis_t aux, double* PQ) {
    const Basis& b = *aux;
    int ns = static_cast<int>(b.sh.size());
    int n = b.nbf;
    std::vector<std::pair<int, int>> pairs;
    for (int i = 0; i < ns; ++i)
        for (int j = 0; j <= i; ++j) pairs.emplace_back(i, j);
#pragma omp parallel
    {
        Scratch s;
        std::vector<double> blk, tmp;
#pragma omp for schedule(dynamic)
        for (size_t k = 0; k < pairs.size(); ++k) {
            const Shell& A = b.sh[pairs[k].first];
            const Shell& C = b.sh[pairs[k].second];
            Shell uA = unit_shell(A.O), uC = unit_shell(C.O);
            blk.resize(static_cast<size_t>(A.ncart) * C.ncart);
            eri_cart(A, uA, C, uC, s, blk.data(), 0, nullptr);
            pure2(b, A, C, blk, tmp);
            for (int i = 0; i < A.nfunc; ++i)
                for (int j = 0; j < C.nfunc; ++j) {
                    double v = blk[i * C.nfunc + j];
                    PQ[static_cast<size_t>(A.off + i) * n + C.off + j] = v;
                    PQ[static_cast<size_t>(C.off + j) * n + A.off + i] = v;
                }
        }
    }
    return 0;
}

int gdfints_schwarz(gdfints_basis_t bp, double* fun_max, double* shell_max) {
    const Basis& b = *bp;
    int ns = static_cast<int>(b.sh.size());
    int n = b.nbf;
    std::vector<std::pair<int, int>> pairs;
    for (int i = 0; i < ns; ++i)
        for (int j = 0; j <= i; ++j) pairs.emplace_back(i, j);
    std::fill(fun_max, fun_max + static_cast<size_t>(n) * n, 0.0);
    std::fill(shell_max, shell_max + static_cast<size_t>(ns) * ns, 0.0);
#pragma omp parallel
    {
        Scratch s;
        std::vector<double> blk, tmp;
#pragma omp for schedule(dynamic)
        for (size_t k = 0; k < pairs.size(); ++k) {
            int M = pairs[k].first, N = pairs[k].second;
            const Shell& A = b.sh[M];
            const Shell& B = b.sh[N];
            blk.resize(static_cast<size_t>(A.ncart) * B.ncart * A.ncart * B.ncart);
            eri_cart(A, B, A, B, s, blk.data(), 0, nullptr);
            int ls[4] = {A.l, B.l, A.l, B.l};
            int pf[4] = {b.puream, b.puream, b.puream, b.puream};
            finish_block(ls, pf, 4, blk, tmp);
            int nm = A.nfunc, nn = B.nfunc;
            double smax = 0.0;
            for (int i = 0; i < nm; ++i)
                for (int j = 0; j < nn; ++j) {
                    int om = A.off + i, on = B.off + j;
                    if (om < on) continue;  // psi4 keeps m >= n only (dfhelper.cc:352)
                    double v = std::fabs(blk[((static_cast<size_t>(i) * nn + j) * nm + i) * nn + j]);
                    smax = std::max(smax, v);
                    fun_max[static_cast<size_t>(om) * n + on] = v;
                    fun_max[static_cast<size_t>(on) * n + om] = v;
                }
            shell_max[static_cast<size_t>(M) * ns + N] = smax;
            shell_max[static_cast<size_t>(N) * ns + M] = smax;
        }
    }
    return 0;
}

}  // extern "C"

namespace {
int three_index_impl(gdfints_basis_t auxp, gdfints_basis_t primp, const unsigned char* shell_mask, int p0, int p1,
                     double omega, double* out) {
    const Basis& aux = *auxp;
    const Basis& pb = *primp;
    int nsp = static_cast<int>(pb.sh.size());
    int nsa = static_cast<int>(aux.sh.size());
    size_t nbf = pb.nbf;
    size_t npair = nbf * (nbf + 1) / 2;
    if (p0 < 0 || p1 > aux.nbf || p0 > p1) return fail("three_index: bad aux range");
    std::vector<std::pair<int, int>> pairs;
    for (int i = 0; i < nsp; ++i)
        for (int j = 0; j <= i; ++j) pairs.emplace_back(i, j);
    std::vector<int> auxsh;
    for (int P = 0; P < nsa; ++P) {
        const Shell& S = aux.sh[P];
        if (S.off + S.nfunc <= p0 || S.off >= p1) continue;
        auxsh.push_back(P);
    }
#pragma omp parallel
    {
        Scratch s;
        std::vector<double> blk, tmp;
#pragma omp for schedule(dynamic)
        for (size_t k = 0; k < pairs.size(); ++k) {
            int M = pairs[k].first, N = pairs[k].second;
            const Shell& A = pb.sh[M];
            const Shell& B = pb.sh[N];
            bool sig = !shell_mask || shell_mask[static_cast<size_t>(M) * nsp + N];
            for (int P : auxsh) {
                const Shell& C = aux.sh[P];
                int nm = A.nfunc, nn = B.nfunc, np = C.nfunc;
                if (sig) {
                    Shell uC = unit_shell(C.O);
                    blk.resize(static_cast<size_t>(A.ncart) * B.ncart * C.ncart);
                    eri_cart(A, B, C, uC, s, blk.data(), 0, nullptr, omega);
                    int ls[3] = {A.l, B.l, C.l};
                    int pf[3] = {pb.puream, pb.puream, aux.puream};
                    finish_block(ls, pf, 3, blk, tmp);
                }
                for (int c = 0; c < np; ++c) {
                    int oq = C.off + c;
                    if (oq < p0 || oq >= p1) continue;
                    double* row = out + static_cast<size_t>(oq - p0) * npair;
                    for (int i = 0; i < nm; ++i)
                        for (int j = 0; j < nn; ++j) {
                            size_t om = A.off + i, on = B.off + j;
                            if (om < on) continue;
                            row[om * (om + 1) / 2 + on] = sig ? blk[(static_cast<size_t>(i) * nn + j) * np + c] : 0.0;
                        }
                }
            }
        }
    }
    return 0;
}
}  // namespace

extern "C" {

int gdfints_three_index(gdfints_basis_t auxp, gdfints_basis_t primp, const unsigned char* shell_mask, int p0, int p1,
                        double* out) {
    return three_index_impl(auxp, primp, shell_mask, p0, p1, 0.0, out);
}

int gdfints_three_index_erf(gdfints_basis_t auxp, gdfints_basis_t primp, const unsigned char* shell_mask, int p0, int p1,
                            double omega, double* out) {
    if (!(omega > 0.0)) return fail("three_index_erf: omega must be positive");
    return three_index_impl(auxp, primp, shell_mask, p0, p1, omega, out);
}

// ------------------------------------------------------------------ gradients
int gdfints_overlap_grad(gdfints_basis_t bp, const double* W, int natom, double* grad) {
    const Basis& b = *bp;
    int ns = static_cast<int>(b.sh.size());
    int n = b.nbf;
    int nt = nthreads();
    std::vector<std::vector<double>> gl(nt, std::vector<double>(3 * natom, 0.0));
#pragma omp parallel
    {
        std::vector<double> blk, dA, tmp, one;
        auto& g = gl[thread_id()];
#pragma omp for schedule(dynamic)
        for (int M = 0; M < ns; ++M)
            for (int N = 0; N < ns; ++N) {
                const Shell& A = b.sh[M];
                const Shell& B = b.sh[N];
                if (A.atom == B.atom) continue;
                one_e_block(A, B, ONE_S, 1, blk, dA);
                size_t nab = static_cast<size_t>(A.ncart) * B.ncart;
                for (int d = 0; d < 3; ++d) {
                    one.assign(dA.begin() + d * nab, dA.begin() + (d + 1) * nab);
                    pure2(b, A, B, one, tmp);
                    double acc = 0.0;
                    for (int i = 0; i < A.nfunc; ++i)
                        for (int j = 0; j < B.nfunc; ++j)
                            acc += W[static_cast<size_t>(A.off + i) * n + B.off + j] * one[i * B.nfunc + j];
                    // d/dA of <a|b> and d/dA of <b|a> are equal: the (N,M) visit adds the B side
                    g[3 * A.atom + d] += 2.0 * acc;
                }
            }
    }
    for (auto& g : gl)
        for (int k = 0; k < 3 * natom; ++k) grad[k] += g[k];
    return 0;
}

int gdfints_kinetic_grad(gdfints_basis_t bp, const double* D, int natom, double* grad) {
    const Basis& b = *bp;
    int ns = static_cast<int>(b.sh.size());
    int n = b.nbf;
    int nt = nthreads();
    std::vector<std::vector<double>> gl(nt, std::vector<double>(3 * natom, 0.0));
#pragma omp parallel
    {
        std::vector<double> blk, dA, tmp, one;
        auto& g = gl[thread_id()];
#pragma omp for schedule(dynamic)
        for (int M = 0; M < ns; ++M)
            for (int N = 0; N < ns; ++N) {
                const Shell& A = b.sh[M];
                const Shell& B = b.sh[N];
                if (A.atom == B.atom) continue;
                one_e_block(A, B, ONE_T, 1, blk, dA);
                size_t nab = static_cast<size_t>(A.ncart) * B.ncart;
                for (int d = 0; d < 3; ++d) {
                    one.assign(dA.begin() + d * nab, dA.begin() + (d + 1) * nab);
                    pure2(b, A, B, one, tmp);
                    double acc = 0.0;
                    for (int i = 0; i < A.nfunc; ++i)
                        for (int j = 0; j < B.nfunc; ++j)
                            acc += D[static_cast<size_t>(A.off + i) * n + B.off + j] * one[i * B.nfunc + j];
                    g[3 * A.atom + d] += 2.0 * acc;
                }
            }
    }
    for (auto& g : gl)
        for (int k = 0; k < 3 * natom; ++k) grad[k] += g[k];
    return 0;
}

int gdfints_potential_grad(gdfints_basis_t bp, const double* D, int natom, const double* Z, const double* xyz,
                           double* grad) {
    const Basis& b = *bp;
    int ns = static_cast<int>(b.sh.size());
    int n = b.nbf;
    int nt = nthreads();
    std::vector<std::vector<double>> gl(nt, std::vector<double>(3 * natom, 0.0));
#pragma omp parallel
    {
        Scratch s;
        std::vector<double> blk, dAB, dC, tmp, one;
        auto& g = gl[thread_id()];
#pragma omp for schedule(dynamic)
        for (int M = 0; M < ns; ++M)
            for (int N = 0; N <= M; ++N) {
                const Shell& A = b.sh[M];
                const Shell& B = b.sh[N];
                potential_block(A, B, natom, Z, xyz, 1, s, blk, dAB, dC);
                size_t nab = static_cast<size_t>(A.ncart) * B.ncart;
                double w = (M == N) ? 1.0 : 2.0;
                auto dot = [&](const double* src) {
                    one.assign(src, src + nab);
                    pure2(b, A, B, one, tmp);
                    double acc = 0.0;
                    for (int i = 0; i < A.nfunc; ++i)
                        for (int j = 0; j < B.nfunc; ++j)
                            acc += D[static_cast<size_t>(A.off + i) * n + B.off + j] * one[i * B.nfunc + j];
                    return w * acc;
                };
                for (int d = 0; d < 3; ++d) {
                    g[3 * A.atom + d] += dot(&dAB[d * nab]);
                    g[3 * B.atom + d] += dot(&dAB[(3 + d) * nab]);
                }
                for (int C = 0; C < natom; ++C)
                    for (int d = 0; d < 3; ++d) g[3 * C + d] += dot(&dC[(3 * C + d) * nab]);
            }
    }
    for (auto& g : gl)
        for (int k = 0; k < 3 * natom; ++k) grad[k] += g[k];
    return 0;
}

int gdfints_metric_grad(gdfints_basis_t auxp, const double* G, int natom, double* grad) {
    const Basis& b = *auxp;
    int ns = static_cast<int>(b.sh.size());
    int n = b.nbf;
    int nt = nthreads();
    std::vector<std::vector<double>> gl(nt, std::vector<double>(3 * natom, 0.0));
#pragma omp parallel
    {
        Scratch s;
        std::vector<double> blk, dblk, one, tmp;
        auto& g = gl[thread_id()];
#pragma omp for schedule(dynamic)
        for (int M = 0; M < ns; ++M)
            for (int N = 0; N < M; ++N) {
                const Shell& A = b.sh[M];
                const Shell& C = b.sh[N];
                if (A.atom == C.atom) continue;
                Shell uA = unit_shell(A.O), uC = unit_shell(C.O);
                size_t nb = static_cast<size_t>(A.ncart) * C.ncart;
                blk.resize(nb);
                dblk.resize(9 * nb);
                eri_cart(A, uA, C, uC, s, blk.data(), 1, dblk.data());
                for (int d = 0; d < 3; ++d) {
                    one.assign(dblk.begin() + d * nb, dblk.begin() + (d + 1) * nb);
                    pure2(b, A, C, one, tmp);
                    double acc = 0.0;
                    for (int i = 0; i < A.nfunc; ++i)
                        for (int j = 0; j < C.nfunc; ++j)
                            acc += G[static_cast<size_t>(A.off + i) * n + C.off + j] * one[i * C.nfunc + j];
                    acc *= 2.0;  // (PQ) and (QP)
                    g[3 * A.atom + d] += acc;
                    g[3 * C.atom + d] -= acc;
                }
            }
    }
    for (auto& g : gl)
        for (int k = 0; k < 3 * natom; ++k) grad[k] += g[k];
    return 0;
}

int gdfints_three_index_grad(gdfints_basis_t auxp, gdfints_basis_t primp, const unsigned char* shell_mask,
                             const double* G3, int natom, double* grad) {
    const Basis& aux = *auxp;
    const Basis& pb = *primp;
    int nsp = static_cast<int>(pb.sh.size());
    int nsa = static_cast<int>(aux.sh.size());
    size_t nbf = pb.nbf;
    size_t npair = nbf * (nbf + 1) / 2;
    std::vector<std::pair<int, int>> pairs;
    for (int i = 0; i < nsp; ++i)
        for (int j = 0; j <= i; ++j)
            if (!shell_mask || shell_mask[static_cast<size_t>(i) * nsp + j]) pairs.emplace_back(i, j);
    int nt = nthreads();
    std::vector<std::vector<double>> gl(nt, std::vector<double>(3 * natom, 0.0));
#pragma omp parallel
    {
        Scratch s;
        std::vector<double> blk, dblk, one, tmp;
        auto& g = gl[thread_id()];
#pragma omp for schedule(dynamic)
        for (size_t k = 0; k < pairs.size(); ++k) {
            int M = pairs[k].first, N = pairs[k].second;
            const Shell& A = pb.sh[M];
            const Shell& B = pb.sh[N];
            for (int P = 0; P < nsa; ++P) {
                const Shell& C = aux.sh[P];
                if (A.atom == B.atom && B.atom == C.atom) continue;
                Shell uC = unit_shell(C.O);
                size_t nb = static_cast<size_t>(A.ncart) * B.ncart * C.ncart;
                blk.resize(nb);
                dblk.resize(9 * nb);
                eri_cart(A, B, C, uC, s, blk.data(), 1, dblk.data());
                int ls[3] = {A.l, B.l, C.l};
                int pf[3] = {pb.puream, pb.puream, aux.puream};
                int nm = A.nfunc, nn = B.nfunc, np = C.nfunc;
                double gA[3] = {0, 0, 0}, gB[3] = {0, 0, 0};
                for (int which = 0; which < 6; ++which) {
                    one.assign(dblk.begin() + which * nb, dblk.begin() + (which + 1) * nb);
                    finish_block(ls, pf, 3, one, tmp);
                    double acc = 0.0;
                    for (int i = 0; i < nm; ++i)
                        for (int j = 0; j < nn; ++j) {
                            size_t om = A.off + i, on = B.off + j;
                            if (om < on) continue;
                            size_t pr = om * (om + 1) / 2 + on;
                            for (int c = 0; c < np; ++c)
                                acc += G3[static_cast<size_t>(C.off + c) * npair + pr] * one[(static_cast<size_t>(i) * nn + j) * np + c];
                        }
                    if (which < 3)
                        gA[which] += acc;
                    else
                        gB[which - 3] += acc;
                }
                for (int d = 0; d < 3; ++d) {
                    g[3 * A.atom + d] += gA[d];
                    g[3 * B.atom + d] += gB[d];
                    g[3 * C.atom + d] -= gA[d] + gB[d];
                }
            }
        }
    }
    for (auto& g : gl)
        for (int k = 0; k < 3 * natom; ++k) grad[k] += g[k];
    return 0;
}

}  // extern "C"
