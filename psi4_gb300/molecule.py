"""Molecules for the DF-JK engine: explicit geometries and the seeded workload generators.

Lengths are converted with psi4's constant ``pc_bohr2angstroms = 0.52917721067``
(psi4 ``include/psi4/physconst.h:402``) so nuclear repulsion energies agree with psi4's.

Seeded generators (the workload configurations the engine is measured on):

* ``water_cluster(nx, ny, nz, seed)`` — one H2O per site of an nx x ny x nz cubic lattice
  of 3.0 Å spacing, each monomer with O-H 0.9572 Å, angle HOH 104.52°, a uniformly random
  SO(3) orientation (normalised quaternion from four N(0,1) draws) and a +/-0.3 Å uniform
  jitter of its position; ``numpy.random.default_rng(seed)``.
* ``linear_alkane(n, seed)`` — all-trans CnH(2n+2) zig-zag with C-C 1.54 Å, C-H 1.09 Å and
  tetrahedral angles, +/-0.02 Å seeded uniform jitter on every atom.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

BOHR2ANGSTROM = 0.52917721067
ANGSTROM2BOHR = 1.0 / BOHR2ANGSTROM

Z_OF = {"H": 1, "He": 2, "Li": 3, "Be": 4, "B": 5, "C": 6, "N": 7, "O": 8, "F": 9, "Ne": 10, "Na": 11, "Mg": 12,
        "Al": 13, "Si": 14, "P": 15, "S": 16, "Cl": 17, "Ar": 18}


@dataclass
class Molecule:
    symbols: list
    xyz: np.ndarray  # (natom, 3) in bohr
    charge: int = 0
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def natom(self) -> int:
        return len(self.symbols)

    @property
    def Z(self) -> np.ndarray:
        return np.array([Z_OF[s] for s in self.symbols], dtype=np.float64)

    @property
    def nelectron(self) -> int:
        return int(self.Z.sum()) - self.charge

    def nuclear_repulsion_energy(self) -> float:
        Z = self.Z
        e = 0.0
        for i in range(self.natom):
            for j in range(i):
                e += Z[i] * Z[j] / np.linalg.norm(self.xyz[i] - self.xyz[j])
        return float(e)

    def nuclear_repulsion_grad(self) -> np.ndarray:
        Z = self.Z
        g = np.zeros((self.natom, 3))
        for i in range(self.natom):
            for j in range(self.natom):
                if i == j:
                    continue
                d = self.xyz[i] - self.xyz[j]
                r = np.linalg.norm(d)
                g[i] -= Z[i] * Z[j] * d / r**3
        return g

    def displaced(self, atom: int, axis: int, step_bohr: float) -> "Molecule":
        xyz = self.xyz.copy()
        xyz[atom, axis] += step_bohr
        return Molecule(list(self.symbols), xyz, self.charge, self.name, dict(self.meta))

    @staticmethod
    def from_angstrom(symbols, xyz_ang, charge=0, name="") -> "Molecule":
        return Molecule(list(symbols), np.asarray(xyz_ang, dtype=np.float64) * ANGSTROM2BOHR, charge, name)


def zmatrix(lines, name="") -> Molecule:
    """Tiny Z-matrix reader (angstrom/degrees): first atom at the origin, second on +z,
    third in the xz plane, later atoms by bond/angle/dihedral."""
    syms, pos = [], []
    for raw in lines:
        t = raw.split()
        if not t:
            continue
        syms.append(t[0])
        if len(pos) == 0:
            pos.append(np.zeros(3))
        elif len(pos) == 1:
            pos.append(np.array([0.0, 0.0, float(t[2])]))
        else:
            a, r = int(t[1]) - 1, float(t[2])
            b, ang = int(t[3]) - 1, math.radians(float(t[4]))
            if len(pos) == 2:
                # place in the xz plane
                u = pos[b] - pos[a]
                u /= np.linalg.norm(u)
                perp = np.array([1.0, 0.0, 0.0])
                v = math.cos(ang) * u + math.sin(ang) * perp
                pos.append(pos[a] + r * v)
            else:
                c, dih = int(t[5]) - 1, math.radians(float(t[6]))
                bc = pos[b] - pos[c]
                ab = pos[a] - pos[b]
                n = np.cross(bc, ab)
                n /= np.linalg.norm(n)
                ab /= np.linalg.norm(ab)
                m = np.cross(n, ab)
                d2 = np.array([-r * math.cos(ang), r * math.sin(ang) * math.cos(dih), r * math.sin(ang) * math.sin(dih)])
                pos.append(pos[a] + d2[0] * ab + d2[1] * m + d2[2] * n)
    return Molecule.from_angstrom(syms, np.array(pos), name=name)


def water_c2v(r_ang: float, angle_deg: float) -> Molecule:
    """H2O in the yz plane with the C2 axis on z, O first, H at -y then +y, the H atoms
    on the +z side of O (the frame psi4 reports gradients in for this molecule)."""
    half = math.radians(angle_deg) / 2.0
    y = r_ang * math.sin(half)
    z = r_ang * math.cos(half)
    xyz = np.array([[0.0, 0.0, 0.0], [0.0, -y, z], [0.0, y, z]])
    # centre of mass frame (masses of 16O and 1H), as psi4 orients molecules
    m = np.array([15.99491461957, 1.00782503223, 1.00782503223])
    xyz -= (m[:, None] * xyz).sum(0) / m.sum()
    return Molecule.from_angstrom(["O", "H", "H"], xyz, name="h2o")


def _random_rotation(rng) -> np.ndarray:
    q = rng.standard_normal(4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
            [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
            [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
        ]
    )


def water_cluster(nx: int, ny: int, nz: int, seed: int = 0, spacing: float = 3.0, jitter: float = 0.3) -> Molecule:
    rng = np.random.default_rng(seed)
    r, ang = 0.9572, math.radians(104.52)
    mono = np.array(
        [[0.0, 0.0, 0.0], [r * math.sin(ang / 2), 0.0, r * math.cos(ang / 2)], [-r * math.sin(ang / 2), 0.0, r * math.cos(ang / 2)]]
    )
    syms, xyz = [], []
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                R = _random_rotation(rng)
                shift = np.array([i, j, k], dtype=np.float64) * spacing + rng.uniform(-jitter, jitter, 3)
                for s, p in zip("OHH", mono @ R.T + shift):
                    syms.append(s)
                    xyz.append(p)
    mol = Molecule.from_angstrom(syms, np.array(xyz), name=f"(H2O)_{nx * ny * nz}")
    mol.meta = {"generator": "water_cluster", "lattice": [nx, ny, nz], "seed": seed}
    return mol


def linear_alkane(n: int, seed: int = 0, jitter: float = 0.02) -> Molecule:
    rng = np.random.default_rng(seed)
    cc, ch = 1.54, 1.09
    tet = math.acos(-1.0 / 3.0)
    dx = cc * math.sin(tet / 2)
    dy = cc * math.cos(tet / 2)

    def carbon(i):  # zig-zag backbone in the xy plane along x
        return np.array([i * dx, (i % 2) * dy, 0.0])

    syms = ["C"] * n
    xyz = [carbon(i) for i in range(n)]
    zax = np.array([0.0, 0.0, 1.0])
    for i in range(n):
        c = carbon(i)
        dprev = (carbon(i - 1) - c) / cc
        dnext = (carbon(i + 1) - c) / cc
        # end carbons: the third hydrogen sits where the chain would continue
        if i == 0:
            syms.append("H")
            xyz.append(c + ch * dprev)
        if i == n - 1:
            syms.append("H")
            xyz.append(c + ch * dnext)
        u = -(dprev + dnext)
        u /= np.linalg.norm(u)
        for sgn in (1.0, -1.0):
            syms.append("H")
            xyz.append(c + ch * (math.cos(tet / 2) * u + sgn * math.sin(tet / 2) * zax))
    xyz = np.array(xyz) + rng.uniform(-jitter, jitter, (len(xyz), 3))
    mol = Molecule.from_angstrom(syms, xyz, name=f"C{n}H{2 * n + 2}")
    mol.meta = {"generator": "linear_alkane", "n": n, "seed": seed}
    return mol
