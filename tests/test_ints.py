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
