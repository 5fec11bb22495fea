/*
 * gdfints.h — host Gaussian integral provider for the GB300 DF-JK engine.
 *
 * In psi4 the 2- and 3-centre Coulomb integrals that feed the density-fitted J/K
 * build come from libint2 on the host (psi4/src/psi4/lib3index/dfhelper.cc:1284-1347
 * compute_sparse_pQq_blocking_p_symm, psi4/src/psi4/lib3index/fittingmetric.cc:72
 * form_fitting_metric, the Schwarz (mn|mn) pass at dfhelper.cc:299-371).  libint2 is
 * not part of this project, so this library supplies the same integrals, on the
 * host, from its own McMurchie–Davidson implementation (Hermite expansion + Boys
 * function), with psi4's conventions:
 *
 *   - contracted shells normalised as libint2's embed_normalization does
 *     (psi4/src/psi4/libmints/gshell.cc:72-145): the x^l component of every
 *     contracted shell has unit norm;
 *   - real solid harmonics in psi4's default Gaussian ordering m = 0, +1, -1, +2, -2, ...
 *     (psi4/src/psi4/libmints/solidharmonics.cc:196-228), each pure function of unit norm;
 *   - Cartesian components in the standard order (for l: x-power from l down to 0,
 *     then y-power from the remainder down to 0).
 *
 * Every function returns 0 on success and a negative code on error; gdfints_last_error()
 * returns a message for the calling thread.  All matrices are row-major doubles.
 */
#ifndef GDFINTS_H
#define GDFINTS_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct gdfints_basis_s* gdfints_basis_t;

/* Build a basis from shells.  Shell s has angular momentum l[s], nprim[s] primitives
 * (exponents/raw contraction coefficients at exps/coefs + prim_offset[s]) and centre
 * xyz[3*s..3*s+2] in bohr; atom[s] is the index of the atom it sits on.  puream != 0
 * selects spherical functions.  Raw coefficients are normalised inside. */
int gdfints_basis_create(int nshell, const int* l, const int* nprim, const int* prim_offset,
                         const double* exps, const double* coefs, const double* xyz, const int* atom,
                         int puream, gdfints_basis_t* out);
void gdfints_basis_destroy(gdfints_basis_t b);
int gdfints_basis_nbf(gdfints_basis_t b);
/* first function index of each shell (length nshell) */
int gdfints_basis_shell_offsets(gdfints_basis_t b, int* offsets);

/* One-electron integrals (nbf x nbf): overlap, kinetic, nuclear attraction. */
int gdfints_overlap(gdfints_basis_t b, double* S);
int gdfints_kinetic(gdfints_basis_t b, double* T);
int gdfints_potential(gdfints_basis_t b, int natom, const double* Z, const double* xyz, double* V);

/* Coulomb metric (P|Q), naux x naux. */
int gdfints_metric(gdfints_basis_t aux, double* PQ);

/* Schwarz data: fun_max[m*nbf+n] = |(mn|mn)| for every function pair and
 * shell_max[M*nshell+N] = max over the (MN) shell pair (dfhelper.cc:336-366). */
int gdfints_schwarz(gdfints_basis_t b, double* fun_max, double* shell_max);

/* Raw 3-index integrals (P|mn) for m >= n, Q-major packed lower triangle:
 * out[P*npair + m*(m+1)/2 + n], npair = nbf*(nbf+1)/2.  shell_mask (nshell*nshell,
 * nullable) skips insignificant primary shell pairs (their entries are written 0).
 * Aux functions [p0, p1) only are computed (out holds rows p0..p1-1). */
int gdfints_three_index(gdfints_basis_t aux, gdfints_basis_t prim, const unsigned char* shell_mask,
                        int p0, int p1, double* out);

/* The same with the long-range operator erf(omega r)/r, omega > 0 (psi4's erf_eri 3-index
 * integrals (Q|w|mn) of DFHelper::prepare_AO_wK_core, dfhelper.cc:589-699). */
int gdfints_three_index_erf(gdfints_basis_t aux, gdfints_basis_t prim, const unsigned char* shell_mask,
                            int p0, int p1, double omega, double* out);

/* First derivatives, contracted with densities, for the SCF gradient (natom x 3, added
 * into grad):
 *   gdfints_overlap_grad   : sum_mn W_mn dS_mn/dx
 *   gdfints_kinetic_grad   : sum_mn D_mn dT_mn/dx
 *   gdfints_potential_grad : sum_mn D_mn dV_mn/dx   (basis-centre and operator-centre terms)
 *   gdfints_metric_grad    : sum_PQ G_PQ d(P|Q)/dx
 *   gdfints_three_index_grad : sum_{P, m>=n} G3[P*npair + mn] d(P|mn)/dx,
 *       G3 in the same Q-major packed layout as gdfints_three_index (off-diagonal mn
 *       entries carry the weight of both (mn) and (nm)).                          */
int gdfints_overlap_grad(gdfints_basis_t b, const double* W, int natom, double* grad);
int gdfints_kinetic_grad(gdfints_basis_t b, const double* D, int natom, double* grad);
int gdfints_potential_grad(gdfints_basis_t b, const double* D, int natom, const double* Z,
                           const double* xyz, double* grad);
int gdfints_metric_grad(gdfints_basis_t aux, const double* G, int natom, double* grad);
int gdfints_three_index_grad(gdfints_basis_t aux, gdfints_basis_t prim, const unsigned char* shell_mask,
                             const double* G3, int natom, double* grad);

/* Boys function F_0..F_n(T) (exposed for tests). */
int gdfints_boys(int n, double T, double* F);

const char* gdfints_last_error(void);

#ifdef __cplusplus
}
#endif
#endif
