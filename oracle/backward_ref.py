"""ORACLE — CPU reference for the reverse mode of one DF-JK build (test infrastructure).

For the lr-symmetric build (D = C C^T, J = sum_Q B_Q d_Q, K = sum_Q (B_Q C)(B_Q C)^T) and
upstream gradients gJ = dE/dJ, gK = dE/dK, returns dE/dC and dE/dB (B-space 3-index
density, Q-major packed triangle with off-diagonal entries carrying (mn) and (nm)).
Dense einsum formulation, small systems only.  Verified against central finite
differences in tests/test_backward_ref.py.
"""
import numpy as np


def sym(a):
    return 0.5 * (a + a.T)


def jk_forward_dense(B, C):
    D = C @ C.T
    d = np.einsum("qmn,mn->q", B, D)
    J = np.einsum("qmn,q->mn", B, d)
    X = np.einsum("qmn,ni->qmi", B, C)
    K = np.einsum("qmi,qni->mn", X, X)
    return J, K


def jk_backward_dense(B, C, gJ, gK):
    gJ, gK = sym(gJ), sym(gK)
    D = C @ C.T
    d = np.einsum("qmn,mn->q", B, D)
    g = np.einsum("qmn,mn->q", B, gJ)
    X = np.einsum("qmn,ni->qmi", B, C)
    Y = np.einsum("mn,qni->qmi", gK, X)
    G = (gJ[None] * d[:, None, None] + g[:, None, None] * D[None]
         + np.einsum("qmi,ni->qmn", Y, C) + np.einsum("mi,qni->qmn", C, Y))
    nbf = C.shape[0]
    r, c = np.tril_indices(nbf)
    w = np.where(r > c, 2.0, 1.0)
    Gp = G[:, r, c] * w
    Jg = np.einsum("qmn,q->mn", B, g)
    dC = 2.0 * Jg @ C + 2.0 * np.einsum("qmn,qni->mi", B, Y)
    return dC, Gp
