"""Host integral provider: Boys function, normalisation, symmetry, translational invariance."""
import numpy as np
import pytest

from psi4_gb300.ints import boys
from tests.helpers import system


def test_boys_against_quadrature(ints_built):
    mpmath = pytest.importorskip("mpmath")
    mpmath.mp.dps = 30
    worst = 0.0
    for T in [0.0, 1e-9, 0.02, 0.7, 3.3, 11.0, 27.5, 39.9, 40.0, 66.0]:
        F = boys(20, T)
        for n in range(21):
            ex = float(mpmath.quad(lambda t: t ** (2 * n) * mpmath.e ** (-T * t * t), [0, 1]))
            worst = max(worst, abs(F[n] - ex) / ex)
    assert worst < 1e-13


def test_one_electron_properties(ints_built):
    mol, pb, ab, ints, df = system("h2o", "cc-pvtz")
    S, T, V = ints.overlap(), ints.kinetic(), ints.potential()
    assert np.allclose(np.diag(S), 1.0, atol=1e-13)
    for M in (S, T, V):
        assert np.abs(M - M.T).max() < 1e-13
    assert np.linalg.eigvalsh(S).min() > 0
    assert np.linalg.eigvalsh(T).min() > 0


def test_metric_positive_definite(ints_built):
    mol, pb, ab, ints, df = system("o2", "cc-pvtz")
    M = df.metric
    assert np.abs(M - M.T).max() < 1e-12
    assert np.linalg.eigvalsh(M).min() > 0


def test_nuclear_repulsion_golden():
    from tests.helpers import reference_values
    from psi4_gb300.molecule import zmatrix

    ref = reference_values()
    for key in ("scf2", "scf5_singlet_df"):
        mol = zmatrix(ref[key]["zmatrix"])
        assert abs(mol.nuclear_repulsion_energy() - ref[key]["nuclear_repulsion"]) < 1e-9


def test_erf_three_index_large_omega_is_coulomb(ints_built):
    """erf(w r)/r -> 1/r: at w = 1e6 the long-range 3-index integrals equal the Coulomb ones
    for every angular momentum (water cc-pVTZ: up to f primary, g fitting functions); the
    difference is ~pi/w^2 times an overlap."""
    mol, pb, ab, ints, df = system("h2o", "cc-pvtz")
    A = ints.three_index(shell_mask=df.sparsity.shell_mask)
    W = ints.three_index_erf(1e6, shell_mask=df.sparsity.shell_mask)
    assert np.abs(W - A).max() < 1e-10 * np.abs(A).max()
    W1 = ints.three_index_erf(0.3, shell_mask=df.sparsity.shell_mask)
    assert np.abs(W1 - A).max() > 1e-2  # really attenuated


def test_erf_three_index_gaussian_charges(ints_built):
    """Independent closed form for one-primitive s functions on one centre: two Gaussian
    charges (exponents a1, a2, charges q1, q2) interact through erf(w r)/r as
    q1 q2 2 mu / sqrt(pi) with 1/mu^2 = 1/a1 + 1/a2 + 1/w^2 (w -> inf: the Coulomb case)."""
    from psi4_gb300.basis import BasisSet
    from psi4_gb300.ints import Integrals
    from psi4_gb300.molecule import zmatrix

    mol = zmatrix(["H", "H 1 0.74"])
    pb = BasisSet.build(mol, "cc-pvdz")
    ab = BasisSet.fitting_for(mol, pb)
    ints = Integrals(mol, pb, ab)

    def single_s(bs, atom):
        out = []
        for sh in range(bs.nshell):
            if bs.l[sh] == 0 and bs.nprim[sh] == 1 and bs.atom[sh] == atom:
                out.append((int(bs.shell_offsets[sh]), float(bs.exps[bs.prim_offset[sh]])))
        return out

    m, zeta = single_s(pb, 0)[0]
    aux = single_s(ab, 0)
    assert aux
    pair = m * (m + 1) // 2 + m
    checked = 0
    for omega in (None, 0.4, 1.3):
        V = ints.three_index() if omega is None else ints.three_index_erf(omega)
        for P, zp in aux:
            a1, a2 = 2.0 * zeta, zp  # |phi_m|^2 has charge 1; phi_P charge (2 zp/pi)^(3/4) (pi/zp)^(3/2)
            q2 = (2.0 * zp / np.pi) ** 0.75 * (np.pi / zp) ** 1.5
            inv = 1.0 / a1 + 1.0 / a2 + (0.0 if omega is None else 1.0 / omega ** 2)
            ref = q2 * 2.0 / np.sqrt(np.pi) / np.sqrt(inv)
            assert abs(V[P, pair] - ref) < 1e-12 * abs(ref), (omega, P, V[P, pair], ref)
            checked += 1
    assert checked >= 3
