"""Python face of the host integral provider (libgdfints.so, include/gdfints.h).

This stands where psi4's libint2-backed IntegralFactory/MintsHelper sit for the DF-JK
path: one-electron S, T, V, the Coulomb metric (P|Q), the Schwarz diagonal (mn|mn) and
the raw 3-index (P|mn), plus their first derivatives for the SCF gradient.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _native
from .basis import BasisSet
from .molecule import Molecule


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(rc, L):
    if rc != 0:
        raise RuntimeError("gdfints: " + L.gdfints_last_error().decode())


class NativeBasis:
    """Owns a gdfints_basis_t for a BasisSet."""

    def __init__(self, bs: BasisSet):
        self.bs = bs
        self.L = _native.ints_lib()
        self._keep = [np.ascontiguousarray(x) for x in (bs.l, bs.nprim, bs.prim_offset, bs.exps, bs.coefs, bs.centers, bs.atom)]
        h = ctypes.c_void_p()
        l, nprim, off, ex, cf, cen, at = self._keep
        _check(
            self.L.gdfints_basis_create(bs.nshell, _ptr(l), _ptr(nprim), _ptr(off), _ptr(ex), _ptr(cf), _ptr(cen), _ptr(at),
                                        int(bs.puream), ctypes.byref(h)),
            self.L,
        )
        self.h = h
        self.nbf = self.L.gdfints_basis_nbf(h)
        assert self.nbf == bs.nbf

    def __del__(self):
        try:
            if getattr(self, "h", None):
                self.L.gdfints_basis_destroy(self.h)
        except Exception:
            pass


class Integrals:
    """Integrals for one molecule with an orbital basis and (optionally) a fitting basis."""

    def __init__(self, mol: Molecule, primary: BasisSet, aux: BasisSet | None = None):
        self.mol = mol
        self.primary = primary
        self.aux = aux
        self.L = _native.ints_lib()
        self.nb = NativeBasis(primary)
        self.na = NativeBasis(aux) if aux is not None else None

    # ---- one-electron
    def _sq(self, n):
        return np.zeros((n, n))

    def overlap(self):
        S = self._sq(self.nb.nbf)
        _check(self.L.gdfints_overlap(self.nb.h, _ptr(S)), self.L)
        return S

    def kinetic(self):
        T = self._sq(self.nb.nbf)
        _check(self.L.gdfints_kinetic(self.nb.h, _ptr(T)), self.L)
        return T

    def potential(self):
        V = self._sq(self.nb.nbf)
        Z = np.ascontiguousarray(self.mol.Z)
        xyz = np.ascontiguousarray(self.mol.xyz)
        _check(self.L.gdfints_potential(self.nb.h, self.mol.natom, _ptr(Z), _ptr(xyz), _ptr(V)), self.L)
        return V

    # ---- two-electron
    def metric(self):
        n = self.na.nbf
        M = self._sq(n)
        _check(self.L.gdfints_metric(self.na.h, _ptr(M)), self.L)
        return M

    def schwarz(self):
        n = self.nb.nbf
        ns = self.primary.nshell
        fun = np.zeros((n, n))
        sh = np.zeros((ns, ns))
        _check(self.L.gdfints_schwarz(self.nb.h, _ptr(fun), _ptr(sh)), self.L)
        return fun, sh

    def three_index(self, shell_mask: np.ndarray | None = None, p0: int = 0, p1: int | None = None):
        """Raw (P|mn), m >= n, Q-major packed lower triangle: shape (p1-p0, nbf(nbf+1)/2)."""
        n = self.nb.nbf
        p1 = self.na.nbf if p1 is None else p1
        out = np.zeros((p1 - p0, n * (n + 1) // 2))
        mask = None if shell_mask is None else np.ascontiguousarray(shell_mask, dtype=np.uint8)
        _check(
            self.L.gdfints_three_index(self.na.h, self.nb.h, None if mask is None else _ptr(mask), p0, p1, _ptr(out)),
            self.L,
        )
        return out

    def three_index_erf(self, omega: float, shell_mask: np.ndarray | None = None, p0: int = 0, p1: int | None = None):
        """(P|erf(omega r)/r|mn), the long-range 3-index integrals of psi4's wK
        (DFHelper::prepare_AO_wK_core, dfhelper.cc:589-699), same layout as three_index."""
        n = self.nb.nbf
        p1 = self.na.nbf if p1 is None else p1
        out = np.zeros((p1 - p0, n * (n + 1) // 2))
        mask = None if shell_mask is None else np.ascontiguousarray(shell_mask, dtype=np.uint8)
        _check(
            self.L.gdfints_three_index_erf(self.na.h, self.nb.h, None if mask is None else _ptr(mask), p0, p1,
                                           float(omega), _ptr(out)),
            self.L,
        )
        return out

    # ---- gradients (natom x 3)
    def _g(self):
        return np.zeros((self.mol.natom, 3))

    def overlap_grad(self, W):
        g = self._g()
        W = np.ascontiguousarray(W)
        _check(self.L.gdfints_overlap_grad(self.nb.h, _ptr(W), self.mol.natom, _ptr(g)), self.L)
        return g

    def kinetic_grad(self, D):
        g = self._g()
        D = np.ascontiguousarray(D)
        _check(self.L.gdfints_kinetic_grad(self.nb.h, _ptr(D), self.mol.natom, _ptr(g)), self.L)
        return g

    def potential_grad(self, D):
        g = self._g()
        D = np.ascontiguousarray(D)
        Z = np.ascontiguousarray(self.mol.Z)
        xyz = np.ascontiguousarray(self.mol.xyz)
        _check(self.L.gdfints_potential_grad(self.nb.h, _ptr(D), self.mol.natom, _ptr(Z), _ptr(xyz), _ptr(g)), self.L)
        return g

    def metric_grad(self, G):
        g = self._g()
        G = np.ascontiguousarray(G)
        _check(self.L.gdfints_metric_grad(self.na.h, _ptr(G), self.mol.natom, _ptr(g)), self.L)
        return g

    def three_index_grad(self, G3, shell_mask=None):
        g = self._g()
        G3 = np.ascontiguousarray(G3)
        mask = None if shell_mask is None else np.ascontiguousarray(shell_mask, dtype=np.uint8)
        _check(
            self.L.gdfints_three_index_grad(self.na.h, self.nb.h, None if mask is None else _ptr(mask), _ptr(G3),
                                            self.mol.natom, _ptr(g)),
            self.L,
        )
        return g


def boys(n: int, T: float) -> np.ndarray:
    L = _native.ints_lib()
    F = np.zeros(n + 1)
    _check(L.gdfints_boys(n, T, _ptr(F)), L)
    return F
