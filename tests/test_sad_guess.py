"""The SAD guess (psi4's default, libscf_solver/sad.cc) of the RHF driver: the guess density
holds the molecule's electrons, and an SCF started from it converges to the reference's stored
energy in fewer iterations than from the core guess (CPU: oracle JK)."""
import numpy as np

from oracle.dfjk_ref import OracleJK
from psi4_gb300.scf import core_hamiltonian, rhf, sad_guess
from tests.helpers import reference_values, system


def test_sad_density_holds_the_electrons(ints_built):
    mol, pb, ab, ints, df = system("h2o_8", "cc-pvdz")
    Cs = sad_guess(mol, "cc-pvdz")
    D = Cs @ Cs.T  # alpha density
    assert abs(np.vdot(D, ints.overlap()) - mol.nelectron / 2) < 1e-8


def test_sad_started_scf_reaches_the_reference_energy(ints_built):
    ref = reference_values()["scf2"]
    mol, pb, ab, ints, df = system("h2o_scf2", "cc-pvtz")
    jk = OracleJK(df.to_pQq(), df.sparsity, df.nbf, df.naux)
    H, S, nocc, e_nuc = core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy()
    r_core = rhf(jk, H, S, nocc, e_nuc)
    r_sad = rhf(jk, H, S, nocc, e_nuc, guess_density_factor=sad_guess(mol, "cc-pvtz"))
    assert abs(r_sad.energy - ref["energy"]) < ref["tolerance"]
    assert abs(r_sad.energy - r_core.energy) < 1e-9
    assert r_sad.iterations <= r_core.iterations
