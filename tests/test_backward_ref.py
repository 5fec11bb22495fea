"""The oracle's reverse-mode formulas against central finite differences, and the full RHF
gradient (host derivative integrals + oracle Gamma) against the reference's scf6 values."""
import numpy as np
import pytest

from oracle.backward_ref import jk_backward_dense, jk_forward_dense
from tests.helpers import random_orbitals, reference_values, system


def _energy(B, C, gJ, gK):
    J, K = jk_forward_dense(B, C)
    return float(np.vdot(gJ, J) + np.vdot(gK, K))


def test_backward_formulas_fd(ints_built):
    mol, pb, ab, ints, df = system("h2o")
    B = df.dense()
    rng = np.random.default_rng(5)
    C = random_orbitals(df.nbf, 4, 3)
    gJ = rng.standard_normal((df.nbf, df.nbf))
    gK = rng.standard_normal((df.nbf, df.nbf))
    dC, Gp = jk_backward_dense(B, C, gJ, gK)
    h = 1e-5
    for (m, i) in [(0, 0), (5, 2), (23, 3)]:
        Cp, Cm = C.copy(), C.copy()
        Cp[m, i] += h
        Cm[m, i] -= h
        fd = (_energy(B, Cp, gJ, gK) - _energy(B, Cm, gJ, gK)) / (2 * h)
        assert abs(fd - dC[m, i]) < 1e-6 * max(1.0, abs(fd))
    r, c = np.tril_indices(df.nbf)
    for (Q, p) in [(0, 0), (3, 17), (50, 200), (115, 299)]:
        m, n = r[p], c[p]
        Bp, Bm = B.copy(), B.copy()
        for X, s in ((Bp, h), (Bm, -h)):
            X[Q, m, n] += s
            if m != n:
                X[Q, n, m] += s
        fd = (_energy(Bp, C, gJ, gK) - _energy(Bm, C, gJ, gK)) / (2 * h)
        assert abs(fd - Gp[Q, p]) < 1e-6 * max(1.0, abs(fd))


def test_rhf_gradient_scf6_golden(ints_built):
    """tests/scf6/input.dat: DF-RHF water cc-pVDZ gradient, compared to 1e-5 there."""
    from oracle.dfjk_ref import OracleJK
    from psi4_gb300.grad import rhf_gradient
    from psi4_gb300.scf import core_hamiltonian, rhf

    ref = reference_values()["scf6_rhf_gradient"]
    mol, pb, ab, ints, df = system("h2o_c2v", "cc-pvdz")
    jk = OracleJK(df.to_pQq(), df.sparsity, df.nbf, df.naux)
    res = rhf(jk, core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy(),
              e_conv=1e-10, d_conv=1e-10)
    C = res.C[:, : res.nocc]
    D = C @ C.T
    _, Gamma = jk_backward_dense(df.dense(), C, 2.0 * D, -D)
    g = rhf_gradient(mol, ints, df, res, Gamma)
    ref_g = np.array(ref["gradient"])
    assert np.abs(g - ref_g).max() < ref["tolerance"], (g, ref_g)
    # translational invariance
    assert np.abs(g.sum(0)).max() < 1e-8
