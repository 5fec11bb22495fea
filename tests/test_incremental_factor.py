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


def test_factor_is_small_for_a_small_change():
    """|U|^2 scales with |dD| (the split-precision increment's error is relative to it): a
    change 1e-6 in the orbitals gives a factor of norm ~1e-3, as the eigendecomposition would."""
    rng = np.random.default_rng(5)
    nbf, nocc = 120, 20
    C1 = np.linalg.qr(rng.standard_normal((nbf, nocc)))[0]
    for eps in (1e-2, 1e-6):
        C2 = C1 + eps * rng.standard_normal((nbf, nocc))
        U, npos = density_difference_factor(C2, C1)
        dD = C2 @ C2.T - C1 @ C1.T
        rec = U[:, :npos] @ U[:, :npos].T - U[:, npos:] @ U[:, npos:].T
        assert np.abs(rec - dD).max() < 1e-13 * max(1.0, np.abs(dD).max()) + 1e-15
        assert np.abs(U).max() ** 2 < 100 * np.abs(dD).max()
