// ints3c.cu — the raw 3-index integrals (P|mn) and the Coulomb metric (P|Q) on the GB300.
//
// psi4 computes them on the host with libint2: DFHelper::prepare_AO_core
// (psi4/src/psi4/lib3index/dfhelper.cc:514-588) fills (P|mn) for the Schwarz-significant shell
// pairs through compute_sparse_pQq_blocking_p_symm (:1284-1347), and the metric comes from
// FittingMetric::form_fitting_metric (psi4/src/psi4/lib3index/fittingmetric.cc:72).  Here they
// are computed where B is contracted and stored, so the 3-index tensor never crosses the
// host link.  The method is the McMurchie–Davidson scheme of the host provider
// (Helgaker, Jørgensen & Olsen, "Molecular Electronic-Structure Theory", ch. 9), arranged per
// shell triplet for the FP64 pipes:
//   * one CTA per primary shell pair (A, B) of one angular-momentum class (la >= lb) and
//     group of 64 fitting shells of one class lc; the pair's primitive products (exponent p,
//     centre P, coefficient product) and their 1D Hermite coefficients E^{ij}_t are staged
//     once in shared memory and read by every thread as broadcasts;
//   * one thread per fitting shell C: per primitive triplet the Boys values F_0..F_L
//     (grid + Taylor expansion, downward recursion), the Hermite integrals R_tuv built in
//     place from the highest order down, the fitting Gaussian's Hermite sum for each of its
//     Cartesian components, and the pair's E contracted one dimension at a time;
//   * Cartesian -> solid harmonics in the thread, written straight into the packed-triangle
//     rows out[(P - p0) * ldo + m(m+1)/2 + n] (or a caller's column map).
// Every angular-momentum class is its own template instance, so the loop bounds are
// constants.  The shared tables (component order, solid harmonics, Boys grid, shell
// normalisation) come from ints/gto_tables.h, the same as the host provider's.
#include <cuda_runtime.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "common.cuh"
#include "gdfjk.h"
#include "ints3c.cuh"

struct gdfjk_basis_s {
    int device = 0;
    int nshell = 0, nbf = 0, puream = 1, maxl = 0;
    std::vector<int> l, nprim, poff, foff, atom;
    std::vector<double> xyz;
    int *d_l = nullptr, *d_nprim = nullptr, *d_poff = nullptr, *d_foff = nullptr, *d_atom = nullptr;
    double *d_xyz = nullptr, *d_exps = nullptr, *d_coefs = nullptr;
};

namespace gdfjk {
namespace ints {

int ppw(int la, int lb) { return 5 + 3 * (la + 1) * (lb + 1) * (la + lb + 1); }
int ppw_grad(int la, int lb) { return 7 + 3 * (la + 2) * (lb + 2) * (la + lb + 3); }


Eri3Kernel pick(int la, int lb, int lc) {
    switch (lc) {
        case 0: return pick_lc0(la, lb);
        case 1: return pick_lc1(la, lb);
        case 2: return pick_lc2(la, lb);
        case 3: return pick_lc3(la, lb);
        case 4: return pick_lc4(la, lb);
        default: return nullptr;
    }
}

// Boys grid and solid-harmonic table, once per device
struct DeviceTables {
    double* boys = nullptr;  // Boys grid, then the solid-harmonic matrices
};
std::mutex g_tab_mutex;
std::map<int, DeviceTables> g_tabs;

int device_tables(int device, const double** boys_out, const double** pure_out, std::string& err) {
    std::lock_guard<std::mutex> lk(g_tab_mutex);
    DeviceTables& t = g_tabs[device];
    const size_t nboys = (size_t)gto::boys_ngrid() * BOYS_STRIDE;
    if (!t.boys) {
        std::vector<double> tab = gto::boys_grid(gto::boys_ngrid(), BOYS_STRIDE, gto::BOYS_H);
        for (int l = 0; l <= MAXL_FIT; ++l) {
            const std::vector<double> m = gto::pure_matrix(l);
            tab.insert(tab.end(), m.begin(), m.end());
        }
        if (tab.size() != nboys + PURE_TABLE) {
            err = "integrals: solid-harmonic table size";
            return GDFJK_ERR_ARG;
        }
        void* p = nullptr;
        if (engine_malloc(&p, tab.size() * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            err = "integrals: device allocation of the Boys table refused";
            return GDFJK_ERR_OOM;
        }
        if (cudaMemcpy(p, tab.data(), tab.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
            cudaFree(p);
            err = "integrals: copy of the Boys table failed";
            return GDFJK_ERR_CUDA;
        }
        t.boys = (double*)p;
    }
    *boys_out = t.boys;
    *pure_out = t.boys + nboys;
    return GDFJK_OK;
}

Shells shells_of(const gdfjk_basis_s* b) {
    return Shells{b->d_atom, b->d_l, b->d_nprim, b->d_poff, b->d_foff, b->d_xyz, b->d_exps, b->d_coefs};
}

// device copies of the class lists of one call, released on return
struct ListBuffers {
    std::vector<void*> p;
    ~ListBuffers() {
        for (void* q : p) cudaFree(q);
    }
    template <class T>
    int upload(const std::vector<T>& v, T** out, std::string& err) {
        void* d = nullptr;
        if (engine_malloc(&d, std::max<size_t>(16, v.size() * sizeof(T))) != cudaSuccess) {
            cudaGetLastError();
            err = "integrals: device allocation of the shell lists refused";
            return GDFJK_ERR_OOM;
        }
        p.push_back(d);
        if (!v.empty() && cudaMemcpy(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice) != cudaSuccess) {
            err = "integrals: copy of the shell lists failed";
            return GDFJK_ERR_CUDA;
        }
        *out = (T*)d;
        return GDFJK_OK;
    }
};

// Launch every class: pairs grouped by (la, lb), fitting shells by lc.
int run_classes(const gdfjk_basis_s* ab, const gdfjk_basis_s* cs, const std::vector<int2>* pair_cls, int npair_cls,
                const std::vector<int>* fit_cls, Eri3Args base, cudaStream_t stream, std::string& err) {
    const double *boys = nullptr, *pure = nullptr;
    int rc = device_tables(ab->device, &boys, &pure, err);
    if (rc) return rc;
    base.boys = boys;
    base.pure = pure;
    base.ab = shells_of(ab);
    base.cs = shells_of(cs);
    ListBuffers lists;
    for (int pc = 0; pc < npair_cls; ++pc) {
        const std::vector<int2>& pl = pair_cls[pc];
        if (pl.empty()) continue;
        const int la = ab->l[pl[0].x], lb = pl[0].y < 0 ? 0 : ab->l[pl[0].y];
        int max_pp = 1;
        for (const int2& q : pl) max_pp = std::max(max_pp, ab->nprim[q.x] * (q.y < 0 ? 1 : ab->nprim[q.y]));
        const size_t smem = (size_t)max_pp * ppw(la, lb) * sizeof(double);
        int2* d_pairs = nullptr;
        if ((rc = lists.upload(pl, &d_pairs, err))) return rc;
        for (int lc = 0; lc <= MAXL_FIT; ++lc) {
            const std::vector<int>& fl = fit_cls[lc];
            if (fl.empty()) continue;
            Eri3Kernel k = pick(la, lb, lc);
            if (!k) {
                err = "integrals: no kernel for the angular momenta (" + std::to_string(la) + " " + std::to_string(lb) +
                      " | " + std::to_string(lc) + ")";
                return GDFJK_ERR_ARG;
            }
            if (smem > 48 * 1024) {
                if (smem > 200 * 1024) {
                    err = "integrals: too many primitive products in one shell pair";
                    return GDFJK_ERR_ARG;
                }
                cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            }
            int* d_fits = nullptr;
            if ((rc = lists.upload(fl, &d_fits, err))) return rc;
            Eri3Args args = base;
            args.pairs = d_pairs;
            args.fits = d_fits;
            args.nfit = (int)fl.size();
            const dim3 grid((unsigned)pl.size(), (unsigned)((fl.size() + ERI_THREADS - 1) / ERI_THREADS));
            k<<<grid, ERI_THREADS, smem, stream>>>(args);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                err = std::string("integrals: launch failed: ") + cudaGetErrorString(e);
                return GDFJK_ERR_CUDA;
            }
        }
    }
    cudaError_t e = cudaStreamSynchronize(stream);  // the lists are released on return
    if (e != cudaSuccess) {
        err = std::string("integrals: ") + cudaGetErrorString(e);
        return GDFJK_ERR_CUDA;
    }
    return GDFJK_OK;
}

Eri3GradKernel pick_grad(int la, int lb, int lc) {
    switch (lc) {
        case 0: return pick_grad_lc0(la, lb);
        case 1: return pick_grad_lc1(la, lb);
        case 2: return pick_grad_lc2(la, lb);
        case 3: return pick_grad_lc3(la, lb);
        case 4: return pick_grad_lc4(la, lb);
        default: return nullptr;
    }
}

// The derivative classes, as run_classes; the gradient is accumulated with atomics.
int run_grad_classes(const gdfjk_basis_s* ab, const gdfjk_basis_s* cs, const std::vector<int2>* pair_cls,
                     int npair_cls, const std::vector<int>* fit_cls, Eri3GradArgs base, cudaStream_t stream,
                     std::string& err) {
    const double *boys = nullptr, *pure = nullptr;
    int rc = device_tables(ab->device, &boys, &pure, err);
    if (rc) return rc;
    base.boys = boys;
    base.pure = pure;
    base.ab = shells_of(ab);
    base.cs = shells_of(cs);
    ListBuffers lists;
    for (int pc = 0; pc < npair_cls; ++pc) {
        const std::vector<int2>& pl = pair_cls[pc];
        if (pl.empty()) continue;
        const int la = ab->l[pl[0].x], lb = pl[0].y < 0 ? 0 : ab->l[pl[0].y];
        int max_pp = 1;
        for (const int2& q : pl) max_pp = std::max(max_pp, ab->nprim[q.x] * (q.y < 0 ? 1 : ab->nprim[q.y]));
        const size_t smem = (size_t)max_pp * ppw_grad(la, lb) * sizeof(double);
        int2* d_pairs = nullptr;
        if ((rc = lists.upload(pl, &d_pairs, err))) return rc;
        for (int lc = 0; lc <= MAXL_FIT; ++lc) {
            const std::vector<int>& fl = fit_cls[lc];
            if (fl.empty()) continue;
            Eri3GradKernel k = pick_grad(la, lb, lc);
            if (!k) {
                err = "integral derivatives: no kernel for the angular momenta (" + std::to_string(la) + " " +
                      std::to_string(lb) + " | " + std::to_string(lc) + ")";
                return GDFJK_ERR_ARG;
            }
            if (smem > 40 * 1024) {
                if (smem > 200 * 1024) {
                    err = "integral derivatives: too many primitive products in one shell pair";
                    return GDFJK_ERR_ARG;
                }
                cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
            }
            int* d_fits = nullptr;
            if ((rc = lists.upload(fl, &d_fits, err))) return rc;
            Eri3GradArgs args = base;
            args.pairs = d_pairs;
            args.fits = d_fits;
            args.nfit = (int)fl.size();
            const dim3 grid((unsigned)pl.size(), (unsigned)((fl.size() + ERI_THREADS - 1) / ERI_THREADS));
            k<<<grid, ERI_THREADS, smem, stream>>>(args);
            cudaError_t e = cudaGetLastError();
            if (e != cudaSuccess) {
                err = std::string("integral derivatives: launch failed: ") + cudaGetErrorString(e);
                return GDFJK_ERR_CUDA;
            }
        }
    }
    cudaError_t e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        err = std::string("integral derivatives: ") + cudaGetErrorString(e);
        return GDFJK_ERR_CUDA;
    }
    return GDFJK_OK;
}

bool atoms_valid(const gdfjk_basis_s* b, int natom) {
    for (int a : b->atom)
        if (a < 0 || a >= natom) return false;
    return true;
}

}  // namespace ints
}  // namespace gdfjk

using namespace gdfjk;

extern "C" {

int gdfjk_basis_create(int device, int nshell, const int* l, const int* nprim, const int* prim_offset, const double* exps,
                       const double* coefs, const double* xyz, const int* atom, int puream, gdfjk_basis_t* out) {
    if (!out || nshell <= 0 || !l || !nprim || !prim_offset || !exps || !coefs || !xyz)
        return report_error(GDFJK_ERR_ARG, "basis_create: null argument or no shells");
    auto* b = new gdfjk_basis_s();
    b->device = device;
    b->nshell = nshell;
    b->puream = puream ? 1 : 0;
    int nprim_total = 0;
    for (int s = 0; s < nshell; ++s) {
        if (l[s] < 0 || l[s] > ints::MAXL_FIT || nprim[s] <= 0 || prim_offset[s] < 0) {
            delete b;
            return report_error(GDFJK_ERR_ARG, "basis_create: shell " + std::to_string(s) +
                                                   " has an angular momentum above g or no primitives");
        }
        nprim_total = std::max(nprim_total, prim_offset[s] + nprim[s]);
    }
    std::vector<double> c(coefs, coefs + nprim_total);
    int off = 0;
    for (int s = 0; s < nshell; ++s) {
        gto::normalise_shell(l[s], nprim[s], exps + prim_offset[s], c.data() + prim_offset[s]);
        b->l.push_back(l[s]);
        b->atom.push_back(atom ? atom[s] : -1);
        b->nprim.push_back(nprim[s]);
        b->poff.push_back(prim_offset[s]);
        b->foff.push_back(off);
        off += b->puream ? 2 * l[s] + 1 : ints::ncart(l[s]);
        b->maxl = std::max(b->maxl, l[s]);
    }
    b->nbf = off;
    b->xyz.assign(xyz, xyz + 3 * (size_t)nshell);
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(device);
    auto up = [&](void** d, const void* h, size_t bytes) {
        if (engine_malloc(d, std::max<size_t>(bytes, 16)) != cudaSuccess) return false;
        return cudaMemcpy(*d, h, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
    };
    const bool ok = up((void**)&b->d_l, b->l.data(), nshell * sizeof(int)) &&
                    up((void**)&b->d_atom, b->atom.data(), nshell * sizeof(int)) &&
                    up((void**)&b->d_nprim, b->nprim.data(), nshell * sizeof(int)) &&
                    up((void**)&b->d_poff, b->poff.data(), nshell * sizeof(int)) &&
                    up((void**)&b->d_foff, b->foff.data(), nshell * sizeof(int)) &&
                    up((void**)&b->d_xyz, b->xyz.data(), 3 * (size_t)nshell * sizeof(double)) &&
                    up((void**)&b->d_exps, exps, (size_t)nprim_total * sizeof(double)) &&
                    up((void**)&b->d_coefs, c.data(), (size_t)nprim_total * sizeof(double));
    cudaSetDevice(cur);
    if (!ok) {
        cudaGetLastError();
        gdfjk_basis_destroy(b);
        return report_error(GDFJK_ERR_OOM, "basis_create: device allocation or copy failed");
    }
    *out = b;
    return GDFJK_OK;
}

void gdfjk_basis_destroy(gdfjk_basis_t b) {
    if (!b) return;
    void* ps[] = {b->d_l, b->d_atom, b->d_nprim, b->d_poff, b->d_foff, b->d_xyz, b->d_exps, b->d_coefs};
    for (void* p : ps)
        if (p) cudaFree(p);
    delete b;
}

int gdfjk_basis_nbf(gdfjk_basis_t b) { return b ? b->nbf : -1; }

int gdfjk_three_index_device(gdfjk_basis_t aux, gdfjk_basis_t prim, const unsigned char* shell_mask, int p0, int p1,
                             const int64_t* col_map, int64_t ldo, double* out, void* stream) {
    if (!aux || !prim || !out) return report_error(GDFJK_ERR_ARG, "three_index_device: null argument");
    if (aux->device != prim->device) return report_error(GDFJK_ERR_ARG, "three_index_device: bases on different devices");
    if (p0 < 0 || p1 > aux->nbf || p0 > p1) return report_error(GDFJK_ERR_ARG, "three_index_device: bad aux range");
    const long long npair = (long long)prim->nbf * (prim->nbf + 1) / 2;
    if (ldo < (col_map ? 1 : npair)) return report_error(GDFJK_ERR_ARG, "three_index_device: leading dimension too small");
    if (prim->maxl > ints::MAXL_PAIR)
        return report_error(GDFJK_ERR_ARG, "three_index_device: primary shells above f are not supported");
    if (aux->puream != prim->puream)
        return report_error(GDFJK_ERR_ARG, "three_index_device: the two bases must agree on pure/Cartesian");
    if (p0 == p1) return GDFJK_OK;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(prim->device);
    const int nsp = prim->nshell;
    std::vector<int2> pairs[(ints::MAXL_PAIR + 1) * (ints::MAXL_PAIR + 1)];
    for (int M = 0; M < nsp; ++M)
        for (int N = 0; N <= M; ++N) {
            if (shell_mask && !shell_mask[(size_t)M * nsp + N]) continue;
            const int lm = prim->l[M], ln = prim->l[N];
            const int2 pr = lm >= ln ? make_int2(M, N) : make_int2(N, M);
            pairs[std::max(lm, ln) * (ints::MAXL_PAIR + 1) + std::min(lm, ln)].push_back(pr);
        }
    std::vector<int> fits[ints::MAXL_FIT + 1];
    for (int P = 0; P < aux->nshell; ++P) {
        const int f0 = aux->foff[P], nf = aux->puream ? 2 * aux->l[P] + 1 : ints::ncart(aux->l[P]);
        if (f0 + nf <= p0 || f0 >= p1) continue;
        fits[aux->l[P]].push_back(P);
    }
    ints::Eri3Args base{};
    base.pure_ab = prim->puream;
    base.pure_c = aux->puream;
    base.out = out;
    base.ldo = ldo;
    base.p0 = p0;
    base.p1 = p1;
    base.col_map = reinterpret_cast<const long long*>(col_map);
    base.metric = 0;
    std::string err;
    const int rc = ints::run_classes(prim, aux, pairs, (int)(sizeof(pairs) / sizeof(pairs[0])), fits, base,
                                     (cudaStream_t)stream, err);
    cudaSetDevice(cur);
    return rc ? report_error(rc, err) : GDFJK_OK;
}

int gdfjk_metric_device(gdfjk_basis_t aux, int p0, int p1, int64_t ldo, double* out, void* stream) {
    if (!aux || !out) return report_error(GDFJK_ERR_ARG, "metric_device: null argument");
    if (p0 < 0 || p1 > aux->nbf || p0 > p1) return report_error(GDFJK_ERR_ARG, "metric_device: bad row range");
    if (ldo < aux->nbf) return report_error(GDFJK_ERR_ARG, "metric_device: leading dimension below naux");
    if (p0 == p1) return GDFJK_OK;
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(aux->device);
    std::vector<int2> pairs[ints::MAXL_FIT + 1];  // (Q, unit) by l_Q
    for (int Q = 0; Q < aux->nshell; ++Q) pairs[aux->l[Q]].push_back(make_int2(Q, -1));
    std::vector<int> fits[ints::MAXL_FIT + 1];
    for (int P = 0; P < aux->nshell; ++P) {
        const int f0 = aux->foff[P], nf = aux->puream ? 2 * aux->l[P] + 1 : ints::ncart(aux->l[P]);
        if (f0 + nf <= p0 || f0 >= p1) continue;
        fits[aux->l[P]].push_back(P);
    }
    ints::Eri3Args base{};
    base.pure_ab = aux->puream;
    base.pure_c = aux->puream;
    base.out = out;
    base.ldo = ldo;
    base.p0 = p0;
    base.p1 = p1;
    base.col_map = nullptr;
    base.metric = 1;
    std::string err;
    const int rc = ints::run_classes(aux, aux, pairs, ints::MAXL_FIT + 1, fits, base, (cudaStream_t)stream, err);
    cudaSetDevice(cur);
    return rc ? report_error(rc, err) : GDFJK_OK;
}

int gdfjk_three_index_grad_device(gdfjk_basis_t aux, gdfjk_basis_t prim, const unsigned char* shell_mask,
                                  const double* G3, const int64_t* col_map, int64_t ldg, int natom, double* grad,
                                  void* stream) {
    if (!aux || !prim || !G3 || !grad) return report_error(GDFJK_ERR_ARG, "three_index_grad_device: null argument");
    if (aux->device != prim->device)
        return report_error(GDFJK_ERR_ARG, "three_index_grad_device: bases on different devices");
    const long long npair = (long long)prim->nbf * (prim->nbf + 1) / 2;
    if (ldg < (col_map ? 1 : npair)) return report_error(GDFJK_ERR_ARG, "three_index_grad_device: leading dimension too small");
    if (prim->maxl > ints::MAXL_PAIR)
        return report_error(GDFJK_ERR_ARG, "three_index_grad_device: primary shells above f are not supported");
    if (aux->puream != prim->puream)
        return report_error(GDFJK_ERR_ARG, "three_index_grad_device: the two bases must agree on pure/Cartesian");
    if (natom <= 0 || !ints::atoms_valid(prim, natom) || !ints::atoms_valid(aux, natom))
        return report_error(GDFJK_ERR_ARG, "three_index_grad_device: the bases need atom indices below natom");
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(prim->device);
    const int nsp = prim->nshell;
    std::vector<int2> pairs[(ints::MAXL_PAIR + 1) * (ints::MAXL_PAIR + 1)];
    for (int M = 0; M < nsp; ++M)
        for (int N = 0; N <= M; ++N) {
            if (shell_mask && !shell_mask[(size_t)M * nsp + N]) continue;
            const int lm = prim->l[M], ln = prim->l[N];
            const int2 pr = lm >= ln ? make_int2(M, N) : make_int2(N, M);
            pairs[std::max(lm, ln) * (ints::MAXL_PAIR + 1) + std::min(lm, ln)].push_back(pr);
        }
    std::vector<int> fits[ints::MAXL_FIT + 1];
    for (int P = 0; P < aux->nshell; ++P) fits[aux->l[P]].push_back(P);
    ints::Eri3GradArgs base{};
    base.pure_ab = prim->puream;
    base.pure_c = aux->puream;
    base.G = G3;
    base.ldg = ldg;
    base.col_map = reinterpret_cast<const long long*>(col_map);
    base.grad = grad;
    base.metric = 0;
    std::string err;
    const int rc = ints::run_grad_classes(prim, aux, pairs, (int)(sizeof(pairs) / sizeof(pairs[0])), fits, base,
                                          (cudaStream_t)stream, err);
    cudaSetDevice(cur);
    return rc ? report_error(rc, err) : GDFJK_OK;
}

int gdfjk_potential_grad_device(gdfjk_basis_t prim, const double* Dp, int natom, const double* Z, const double* xyz,
                                double* grad, void* stream) {
    if (!prim || !Dp || !Z || !xyz || !grad) return report_error(GDFJK_ERR_ARG, "potential_grad_device: null argument");
    if (prim->maxl > ints::MAXL_PAIR)
        return report_error(GDFJK_ERR_ARG, "potential_grad_device: primary shells above f are not supported");
    if (natom <= 0 || !ints::atoms_valid(prim, natom))
        return report_error(GDFJK_ERR_ARG, "potential_grad_device: the basis needs atom indices below natom");
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(prim->device);
    const int nsp = prim->nshell;
    std::vector<int2> pairs[(ints::MAXL_PAIR + 1) * (ints::MAXL_PAIR + 1)];
    for (int M = 0; M < nsp; ++M)
        for (int N = 0; N <= M; ++N) {
            const int lm = prim->l[M], ln = prim->l[N];
            const int2 pr = lm >= ln ? make_int2(M, N) : make_int2(N, M);
            pairs[std::max(lm, ln) * (ints::MAXL_PAIR + 1) + std::min(lm, ln)].push_back(pr);
        }
    std::vector<int> fits[ints::MAXL_FIT + 1];
    for (int a = 0; a < natom; ++a) fits[0].push_back(a);
    double* dZ = nullptr;
    std::string err;
    int rc = GDFJK_OK;
    if (engine_malloc((void**)&dZ, (size_t)natom * 4 * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        cudaSetDevice(cur);
        return report_error(GDFJK_ERR_OOM, "potential_grad_device: device allocation refused");
    }
    cudaMemcpy(dZ, Z, (size_t)natom * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(dZ + natom, xyz, (size_t)natom * 3 * sizeof(double), cudaMemcpyHostToDevice);
    ints::Eri3GradArgs base{};
    base.pure_ab = prim->puream;
    base.pure_c = 0;
    base.G = Dp;
    base.ldg = 0;  // every charge reads the same density row
    base.col_map = nullptr;
    base.grad = grad;
    base.metric = 0;
    base.charges = dZ;
    base.charge_xyz = dZ + natom;
    rc = ints::run_grad_classes(prim, prim, pairs, (int)(sizeof(pairs) / sizeof(pairs[0])), fits, base,
                                (cudaStream_t)stream, err);
    cudaFree(dZ);
    cudaSetDevice(cur);
    return rc ? report_error(rc, err) : GDFJK_OK;
}

int gdfjk_metric_grad_device(gdfjk_basis_t aux, const double* G2, int64_t ldg, int natom, double* grad, void* stream) {
    if (!aux || !G2 || !grad) return report_error(GDFJK_ERR_ARG, "metric_grad_device: null argument");
    if (ldg < aux->nbf) return report_error(GDFJK_ERR_ARG, "metric_grad_device: leading dimension below naux");
    if (natom <= 0 || !ints::atoms_valid(aux, natom))
        return report_error(GDFJK_ERR_ARG, "metric_grad_device: the basis needs atom indices below natom");
    int cur = 0;
    cudaGetDevice(&cur);
    cudaSetDevice(aux->device);
    std::vector<int2> pairs[ints::MAXL_FIT + 1];
    for (int Q = 0; Q < aux->nshell; ++Q) pairs[aux->l[Q]].push_back(make_int2(Q, -1));
    std::vector<int> fits[ints::MAXL_FIT + 1];
    for (int P = 0; P < aux->nshell; ++P) fits[aux->l[P]].push_back(P);
    ints::Eri3GradArgs base{};
    base.pure_ab = aux->puream;
    base.pure_c = aux->puream;
    base.G = G2;
    base.ldg = ldg;
    base.col_map = nullptr;
    base.grad = grad;
    base.metric = 1;
    std::string err;
    const int rc = ints::run_grad_classes(aux, aux, pairs, ints::MAXL_FIT + 1, fits, base, (cudaStream_t)stream, err);
    cudaSetDevice(cur);
    return rc ? report_error(rc, err) : GDFJK_OK;
}

}  // extern "C"
