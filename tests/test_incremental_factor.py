"""The signed low-rank factor of dD used by the precision form is exact (CPU)."""
import numpy as np

from psi4_gb300.jk import density_difference_factor


def test_factor_reproduces_density_difference():
    rng = np.random.default_rng(3)
    nbf, nocc = 40, 7
    C1 = rng.standard_normal((nbf, nocc))
    C2 = C1 + 1e-3 * rng.standard_normal((nbf, nocc))
    U, npos = density_difference_factor(C2, C1)
    dD = C2 @ C2.T - C1 @ C1.T
    rec = U[:, :npos] @ U[:, :npos].T - U[:, npos:] @ U[:, npos:].T
    assert np.abs(rec - dD).max() < 1e-12
    assert U.shape[1] <= 2 * nocc


def test_factor_of_identical_densities_is_empty():
    rng = np.random.default_rng(4)
    C = rng.standard_normal((30, 5))
    Q, _ = np.linalg.qr(rng.standard_normal((5, 5)))
    U, npos = density_difference_factor(C @ Q, C)  # same density, rotated orbitals
    assert U.shape[1] == 0 or np.abs(U).max() < 1e-6
