"""Gaussian basis sets on a molecule, in psi4's function order.

Functions are ordered atom by atom and, on each atom, shell by shell in the order of the
basis-set file, exactly as psi4's BasisSet builds them (psi4/src/psi4/libmints/basisset.cc).
The fitting basis keeps the orbital basis's spherical/Cartesian choice, as psi4's
``core.BasisSet.build(..., "DF_BASIS_SCF", ..., "JKFIT", name, puream)`` does
(psi4/driver/p4util/python_helpers.py:493-494).
"""
from __future__ import annotations

import json
import os
from dataclasses import dataclass

import numpy as np

from .molecule import Molecule

_DATA = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "basis")


def _load(name: str) -> dict:
    path = os.path.join(_DATA, name.lower() + ".json")
    if not os.path.exists(path):
        raise ValueError(f"basis set {name!r} is not available (have: {sorted(os.listdir(_DATA))})")
    with open(path) as fh:
        return json.load(fh)


@dataclass
class BasisSet:
    name: str
    puream: bool
    l: np.ndarray          # (nshell,) int32
    nprim: np.ndarray      # (nshell,) int32
    prim_offset: np.ndarray  # (nshell,) int32
    exps: np.ndarray       # (nprim_total,)
    coefs: np.ndarray      # raw contraction coefficients
    centers: np.ndarray    # (nshell, 3) bohr
    atom: np.ndarray       # (nshell,) int32

    @property
    def nshell(self) -> int:
        return int(self.l.shape[0])

    @property
    def nfunc_per_shell(self) -> np.ndarray:
        return (2 * self.l + 1) if self.puream else (self.l + 1) * (self.l + 2) // 2

    @property
    def nbf(self) -> int:
        return int(self.nfunc_per_shell.sum())

    @property
    def shell_offsets(self) -> np.ndarray:
        n = self.nfunc_per_shell
        return np.concatenate([[0], np.cumsum(n)[:-1]]).astype(np.int64)

    @property
    def max_am(self) -> int:
        return int(self.l.max())

    @staticmethod
    def build(mol: Molecule, name: str, puream: bool | None = None) -> "BasisSet":
        doc = _load(name)
        pure = doc["puream"] if puream is None else bool(puream)
        ls, nps, offs, ex, cf, cen, at = [], [], [], [], [], [], []
        off = 0
        for ia, sym in enumerate(mol.symbols):
            shells = doc["elements"].get(sym)
            if shells is None:
                raise ValueError(f"basis {name}: no entry for element {sym}")
            for sh in shells:
                ls.append(sh["l"])
                nps.append(len(sh["exps"]))
                offs.append(off)
                off += len(sh["exps"])
                ex.extend(sh["exps"])
                cf.extend(sh["coefs"])
                cen.append(mol.xyz[ia])
                at.append(ia)
        return BasisSet(
            name=name,
            puream=pure,
            l=np.array(ls, dtype=np.int32),
            nprim=np.array(nps, dtype=np.int32),
            prim_offset=np.array(offs, dtype=np.int32),
            exps=np.array(ex, dtype=np.float64),
            coefs=np.array(cf, dtype=np.float64),
            centers=np.array(cen, dtype=np.float64).reshape(-1, 3),
            atom=np.array(at, dtype=np.int32),
        )

    @staticmethod
    def fitting_for(mol: Molecule, orbital: "BasisSet", name: str | None = None) -> "BasisSet":
        """The JKFIT partner of an orbital basis (cc-pVXZ -> cc-pVXZ-JKFIT), same puream."""
        return BasisSet.build(mol, name or (orbital.name.lower() + "-jkfit"), puream=orbital.puream)
