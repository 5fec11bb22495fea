"""ORACLE — CPU restatement of psi4's in-core density-fitted J/K build (test infrastructure).

This module is the checker for the GB300 engine.  Only ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py`` use it; the product never imports it.

It restates, loop for loop over DFHelper's pQq layout, with numpy standing in for the BLAS
calls:

* ``JK::compute_D``                    psi4/src/psi4/libfock/jk.cc:314-354   (D = C_left C_right^T)
* ``DFHelper::compute_J_symm``         psi4/src/psi4/lib3index/dfhelper.cc:3162-3223
* ``DFHelper::compute_J``              psi4/src/psi4/lib3index/dfhelper.cc:3230-3285 (lr non-symmetric)
* ``DFHelper::first_transform_pQq``    psi4/src/psi4/lib3index/dfhelper.cc:2162-2186
* ``DFHelper::compute_K``              psi4/src/psi4/lib3index/dfhelper.cc:3350-3377
* ``MemDFJK::compute_JK``              psi4/src/psi4/libfock/MemDFJK.cc:97-111 (zero, then build)

Parity pin: psi4 itself cannot be built here (libint2 is not vendored), so this oracle is
pinned through the reference's own golden energies (tests/scf2, tests/scf5,
tests/pytests/test_comprehensive_jk_screening.py) and gradient (tests/scf6), reached by
running the RHF driver with this JK on integrals from the host provider; see
tests/test_golden.py.  It is also cross-checked against an independent dense
einsum formulation (tests/test_oracle.py).
"""
from __future__ import annotations

import numpy as np


def compute_D(C_left, C_right=None):
    """jk.cc:351 — D = C_left C_right^T (DGEMM 'N','T')."""
    C_right = C_left if C_right is None else C_right
    if C_left.shape[1] == 0:
        return np.zeros((C_left.shape[0], C_right.shape[0]))
    return C_left @ C_right.T


class RowTables:
    """Per-row significant-column lists of a sparsity, built once (outside any timed region),
    as psi4 builds schwarz_fun_index_ and the symm_* tables once in prepare_sparsity
    (dfhelper.cc:368-420) and its loops then index with them:
      full[k]   significant n of row k, ascending (the columns of B[k] in pQq order)
      sym[k]    the m >= k part (columns symm_ignored_columns[k] .. +symm_small_skips[k])
      wsym[k]   compute_J_symm's density weights on sym[k]: 1 on the diagonal, 2 off it
                (dfhelper.cc:3186-3192)."""

    def __init__(self, sp, nbf):
        self.full = [np.flatnonzero(sp.fun_index[k]) for k in range(nbf)]
        self.sym = [ms[ms >= k] for k, ms in enumerate(self.full)]
        self.wsym = [np.where(ms == k, 1.0, 2.0) for k, ms in enumerate(self.sym)]


def compute_J_symm(Ppq, sp, D, nbf, naux, tables=None):
    """dfhelper.cc:3162-3223 for one density, the whole aux range as one block (bcount=0,
    block_size=naux, AO_core).  Returns J (nbf x nbf).  `tables` (RowTables) replaces the
    per-row index construction by the precomputed lists; the arithmetic is the same."""
    T1 = np.zeros(naux)
    # pass 1: (Qm)(m) -> (Q), rows k, m >= k significant, off-diagonal weight 2
    for k in range(nbf):
        si = int(sp.small_skips[k])
        mi = int(sp.symm_small_skips[k])
        skip = int(sp.symm_ignored_columns[k])
        jump = int(sp.big_skips[k])
        if mi == 0:
            continue
        if tables is None:
            ms = [m for m in range(k, nbf) if sp.fun_index[k, m]]
            Dbuf = np.array([D[k, m] if m == k else 2.0 * D[k, m] for m in ms])
        else:
            Dbuf = D[k, tables.sym[k]] * tables.wsym[k]
        blk = Ppq[jump: jump + naux * si].reshape(naux, si)[:, skip: skip + mi]
        T1 += blk @ Dbuf
    # pass 2: J_km = sum_Q B[k][Q][m] d_Q over the m >= k part, then unpack + symmetrise
    J = np.zeros((nbf, nbf))
    for k in range(nbf):
        si = int(sp.small_skips[k])
        mi = int(sp.symm_small_skips[k])
        skip = int(sp.symm_ignored_columns[k])
        jump = int(sp.big_skips[k])
        if mi == 0:
            continue
        blk = Ppq[jump: jump + naux * si].reshape(naux, si)[:, skip: skip + mi]
        T2 = T1 @ blk
        if tables is None:
            ms = [m for m in range(k, nbf) if sp.fun_index[k, m]]
            for c, m in enumerate(ms):
                if m == k:
                    J[k, k] += T2[c]
                else:
                    J[k, m] += T2[c]
                    J[m, k] += T2[c]
        else:
            ms = tables.sym[k]
            J[k, ms] += T2
            off = ms != k
            J[ms[off], k] += T2[off]
    return J


def compute_J(Ppq, sp, D, nbf, naux):
    """dfhelper.cc:3230-3285: the non-symmetric J (full rows of significant n)."""
    T1 = np.zeros(naux)
    for k in range(nbf):
        si = int(sp.small_skips[k])
        if si == 0:
            continue
        ms = [m for m in range(nbf) if sp.fun_index[k, m]]
        blk = Ppq[int(sp.big_skips[k]): int(sp.big_skips[k]) + naux * si].reshape(naux, si)
        T1 += blk @ D[k, ms]
    J = np.zeros((nbf, nbf))
    for k in range(nbf):
        si = int(sp.small_skips[k])
        if si == 0:
            continue
        ms = [m for m in range(nbf) if sp.fun_index[k, m]]
        blk = Ppq[int(sp.big_skips[k]): int(sp.big_skips[k]) + naux * si].reshape(naux, si)
        J[k, ms] += T1 @ blk
    return J


def first_transform_pQq(Ppq, sp, Cmat, nbf, naux, tables=None):
    """dfhelper.cc:2162-2186: T[k][Q][i] = sum_{m in sig(k)} B[k][Q][m] C[m][i] (the rows of C
    gathered per k, then one DGEMM per row)."""
    nocc = Cmat.shape[1]
    T = np.zeros((nbf, naux, nocc))
    for k in range(nbf):
        si = int(sp.small_skips[k])
        if si == 0:
            continue
        ms = [m for m in range(nbf) if sp.fun_index[k, m]] if tables is None else tables.full[k]
        blk = Ppq[int(sp.big_skips[k]): int(sp.big_skips[k]) + naux * si].reshape(naux, si)
        T[k] = blk @ Cmat[ms, :]
    return T


def compute_K(Ppq, sp, C_left, C_right, nbf, naux, lr_symmetric=True, tables=None):
    """dfhelper.cc:3350-3377: K += T1 T2^T with inner dimension nocc*naux; nocc=0 skips."""
    nocc = C_left.shape[1]
    K = np.zeros((nbf, nbf))
    if nocc == 0:
        return K
    T1 = first_transform_pQq(Ppq, sp, C_left, nbf, naux, tables).reshape(nbf, naux * nocc)
    T2 = T1 if lr_symmetric else first_transform_pQq(Ppq, sp, C_right, nbf, naux, tables).reshape(nbf, naux * nocc)
    K += T1 @ T2.T
    return K


def compute_wK(m1Ppq, wPpq, sp, C_left, C_right, nbf, naux, lr_symmetric=True):
    """dfhelper.cc:3378-3438 (compute_wK): T1 = transform of J^-1 (Q|mn) (m1Ppq) with C_left,
    T2 = transform of (Q|w|mn) (wPpq) with C_right, wK = T1 T2^T over the inner dimension
    nocc*naux; for lr-symmetric densities MemDFJK::compute_JK then hermitivitizes wK
    (MemDFJK.cc:103-108)."""
    nocc = C_left.shape[1]
    wK = np.zeros((nbf, nbf))
    if nocc == 0:
        return wK
    T1 = first_transform_pQq(m1Ppq, sp, C_left, nbf, naux).reshape(nbf, naux * nocc)
    T2 = first_transform_pQq(wPpq, sp, C_left if lr_symmetric else C_right, nbf, naux).reshape(nbf, naux * nocc)
    wK += T1 @ T2.T
    if lr_symmetric:
        wK = 0.5 * (wK + wK.T)
    return wK


class OracleJK:
    """psi4.core.JK-shaped front end over the restatement (MemDFJK semantics)."""

    def __init__(self, Ppq, sparsity, nbf, naux):
        self.Ppq = np.asarray(Ppq, dtype=np.float64)
        self.sp = sparsity
        self.nbf, self.naux = nbf, naux
        self.do_J = True
        self.do_K = True
        self._Cl, self._Cr = [], []
        self._J, self._K, self._D = [], [], []

    def name(self):
        return "OracleMemDFJK"

    def initialize(self):
        pass

    def set_do_J(self, v):
        self.do_J = bool(v)

    def set_do_K(self, v):
        self.do_K = bool(v)

    def C_clear(self):
        self._Cl, self._Cr = [], []

    def C_left_add(self, C):
        self._Cl.append(np.asarray(C, dtype=np.float64))

    def C_right_add(self, C):
        self._Cr.append(np.asarray(C, dtype=np.float64))

    def C_add(self, C):
        self.C_left_add(C)
        self.C_right_add(C)

    def compute(self):
        lr_symmetric = len(self._Cr) == 0  # jk.cc:597-599
        Cr = self._Cl if lr_symmetric else self._Cr
        self._D = [compute_D(l, r) for l, r in zip(self._Cl, Cr)]
        self._J, self._K = [], []
        for l, r, D in zip(self._Cl, Cr, self._D):
            if self.do_J:
                Jf = compute_J_symm if lr_symmetric else compute_J
                self._J.append(Jf(self.Ppq, self.sp, D, self.nbf, self.naux))
            if self.do_K:
                self._K.append(compute_K(self.Ppq, self.sp, l, r, self.nbf, self.naux, lr_symmetric))

    def J(self):
        return self._J

    def K(self):
        return self._K

    def D(self):
        return self._D


def dense_jk(B_dense, D, C_left=None, C_right=None):
    """Independent dense formulation used to cross-check the loop restatement:
    J_mn = sum_Q B_Qmn (sum_ls B_Qls D_ls), K_mn = sum_Q (B_Q C_l)(B_Q C_r)^T."""
    d = np.einsum("qls,ls->q", B_dense, D)
    J = np.einsum("qmn,q->mn", B_dense, d)
    K = None
    if C_left is not None:
        C_right = C_left if C_right is None else C_right
        Xl = np.einsum("qmn,ni->qmi", B_dense, C_left)
        Xr = np.einsum("qmn,ni->qmi", B_dense, C_right)
        K = np.einsum("qmi,qni->mn", Xl, Xr)
    return J, K


def memdfjk_memory_estimate(sparsity, nbf, naux, qshell_max, nthreads=1):
    """MemDFJK::memory_estimate (psi4/src/psi4/libfock/MemDFJK.cc:65-69) -> DFHelper::get_core_size
    -> AO_core (psi4/src/psi4/lib3index/dfhelper.cc:216-236), in doubles, for the STORE path
    without wK: the sparse AO tensor (big_skips[nbf] = naux * significant pairs), the metric,
    one nbf^2 C buffer per thread and three nbf^2 * Qshell_max temporaries (Qshell_max = the
    most functions in one aux shell, dfhelper.cc:92)."""
    return int(sparsity.big_skips[nbf]) + naux * naux + nthreads * nbf * nbf + 3 * nbf * nbf * qshell_max
