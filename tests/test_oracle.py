"""The oracle's loop restatement of DFHelper (pQq layout) against an independent dense
formulation, on the cases the reference's own JK tests use (tests/pytests/test_dfjk.py:
random non-symmetric C pairs of 16-30 columns, water cc-pVDZ / cc-pVDZ-jkfit)."""
import numpy as np
import pytest

from oracle import dfjk_ref
from tests.helpers import random_orbitals, system


def _dense_with_mask(df):
    return df.dense()


@pytest.mark.parametrize("sizes", [(16, 16), (16, 20), (20, 20), (30, 30)])
def test_loop_restatement_matches_dense(ints_built, sizes):
    mol, pb, ab, ints, df = system("h2o")
    nbf, naux = df.nbf, df.naux
    Ppq = df.to_pQq()
    Bd = _dense_with_mask(df)
    Cl = random_orbitals(nbf, sizes[0], 1)
    Cr = random_orbitals(nbf, sizes[0], 2)
    # lr-symmetric
    D = dfjk_ref.compute_D(Cl)
    J = dfjk_ref.compute_J_symm(Ppq, df.sparsity, D, nbf, naux)
    K = dfjk_ref.compute_K(Ppq, df.sparsity, Cl, Cl, nbf, naux, True)
    Jd, Kd = dfjk_ref.dense_jk(Bd, D, Cl)
    assert np.abs(J - Jd).max() < 1e-11
    assert np.abs(K - Kd).max() < 1e-11
    # non-symmetric pair
    D2 = dfjk_ref.compute_D(Cl, Cr)
    J2 = dfjk_ref.compute_J(Ppq, df.sparsity, D2, nbf, naux)
    K2 = dfjk_ref.compute_K(Ppq, df.sparsity, Cl, Cr, nbf, naux, False)
    Jd2, Kd2 = dfjk_ref.dense_jk(Bd, D2, Cl, Cr)
    assert np.abs(J2 - Jd2).max() < 1e-11
    assert np.abs(K2 - Kd2).max() < 1e-11


def test_screened_layout_and_jk(ints_built):
    # two waters 9 A apart with a loose cutoff: many pairs are screened out
    mol, pb, ab, ints, df = system("h2o_2_far", cutoff=1e-5)
    sp = df.sparsity
    assert 0.0 < sp.sparsity < 1.0
    nbf, naux = df.nbf, df.naux
    Ppq = df.to_pQq()
    # layout formula: Ppq[big_skips[m] + Q*small_skips[m] + fun_index[m,n]-1] = B[Q,m,n]
    rng = np.random.default_rng(0)
    Bd = df.dense()
    for _ in range(200):
        m, n, Q = rng.integers(nbf), rng.integers(nbf), rng.integers(naux)
        if sp.fun_index[m, n]:
            idx = sp.big_skips[m] + Q * sp.small_skips[m] + sp.fun_index[m, n] - 1
            assert Ppq[idx] == Bd[Q, m, n]
    C = random_orbitals(nbf, 10, 4)
    D = dfjk_ref.compute_D(C)
    J = dfjk_ref.compute_J_symm(Ppq, sp, D, nbf, naux)
    K = dfjk_ref.compute_K(Ppq, sp, C, C, nbf, naux, True)
    Jd, Kd = dfjk_ref.dense_jk(Bd, D, C)
    assert np.abs(J - Jd).max() < 1e-11
    assert np.abs(K - Kd).max() < 1e-11


def test_nocc_zero_skips_K(ints_built):
    mol, pb, ab, ints, df = system("h2o")
    C = np.zeros((df.nbf, 0))
    K = dfjk_ref.compute_K(df.to_pQq(), df.sparsity, C, C, df.nbf, df.naux)
    assert not K.any()


def test_oracle_jk_object(ints_built):
    mol, pb, ab, ints, df = system("h2o")
    jk = dfjk_ref.OracleJK(df.to_pQq(), df.sparsity, df.nbf, df.naux)
    C = random_orbitals(df.nbf, 5, 9)
    jk.C_left_add(C)
    jk.compute()
    Jd, Kd = dfjk_ref.dense_jk(df.dense(), C @ C.T, C)
    assert np.abs(jk.J()[0] - Jd).max() < 1e-11
    assert np.abs(jk.K()[0] - Kd).max() < 1e-11
    assert np.abs(jk.D()[0] - C @ C.T).max() < 1e-14


def test_oracle_wk_against_dense(ints_built):
    """compute_wK (DFHelper's loop over its pQq layout) against a dense restatement with
    full square tensors: wK = sum_Q (M1_Q C_l)(W_Q C_r)^T, hermitivitized when lr-symmetric."""
    from oracle import dfjk_ref
    from psi4_gb300.dfhelper import build_wk_tensors
    from tests.helpers import random_orbitals, system

    mol, pb, ab, ints, df = system("h2o", "cc-pvdz")
    m1, w = build_wk_tensors(df, ints, 0.4)
    nbf, naux = df.nbf, df.naux
    r, c = np.tril_indices(nbf)

    def square(tri):
        full = np.zeros((naux, nbf, nbf))
        full[:, r, c] = tri
        full[:, c, r] = tri
        return full

    M1, W = square(m1.B_tri), square(w.B_tri)
    Cl = random_orbitals(nbf, 5, seed=1)
    Cr = random_orbitals(nbf, 5, seed=2)
    dense = np.einsum("qmn,ni,qlk,ki->ml", M1, Cl, W, Cr)
    got = dfjk_ref.compute_wK(m1.to_pQq(), w.to_pQq(), df.sparsity, Cl, Cr, nbf, naux, lr_symmetric=False)
    assert np.abs(got - dense).max() < 1e-12 * max(1.0, np.abs(dense).max())
    sym = np.einsum("qmn,ni,qlk,ki->ml", M1, Cl, W, Cl)
    got = dfjk_ref.compute_wK(m1.to_pQq(), w.to_pQq(), df.sparsity, Cl, None, nbf, naux)
    assert np.abs(got - 0.5 * (sym + sym.T)).max() < 1e-12 * max(1.0, np.abs(sym).max())


def test_row_tables_give_the_same_results(ints_built):
    """The precomputed per-row index lists (RowTables, used by the timed CPU baseline) give
    bitwise the loop restatement's J and K, on a screened layout."""
    mol, pb, ab, ints, df = system("h2o_2_far", cutoff=1e-5)
    sp = df.sparsity
    nbf, naux = df.nbf, df.naux
    Ppq = df.to_pQq()
    tb = dfjk_ref.RowTables(sp, nbf)
    C = random_orbitals(nbf, 7, 11)
    D = dfjk_ref.compute_D(C)
    assert np.array_equal(dfjk_ref.compute_J_symm(Ppq, sp, D, nbf, naux),
                          dfjk_ref.compute_J_symm(Ppq, sp, D, nbf, naux, tb))
    assert np.array_equal(dfjk_ref.compute_K(Ppq, sp, C, C, nbf, naux, True),
                          dfjk_ref.compute_K(Ppq, sp, C, C, nbf, naux, True, tb))
