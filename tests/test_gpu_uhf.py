"""UHF on the GPU engine: two lr-symmetric densities per build (alpha, beta) through
GpuDFJK, native FP64 and the emulated-FP64 form, against the reference's triplet-O2 DF
energy and the oracle's per-iteration J/K."""
import numpy as np
import pytest

from oracle import dfjk_ref
from psi4_gb300.jk import GpuDFJK
from psi4_gb300.scf import core_hamiltonian, uhf
from tests.helpers import reference_values, system

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "fp64-emulated"])
def test_uhf_triplet_o2(ints_built, jk_built, precision):
    ref = reference_values()["scf5_triplet_uhf_df"]
    mol, pb, ab, ints, df = system("o2", "cc-pvtz")
    jk = GpuDFJK.from_tensor(df)
    jk.set_precision(precision)
    jk.initialize()
    r = uhf(jk, core_hamiltonian(ints), ints.overlap(), ref["nalpha"], ref["nbeta"], mol.nuclear_repulsion_energy())
    print(f"UHF {precision}: {r.energy:.12f} ref {ref['energy']:.12f} ({r.iterations} iterations)")
    assert abs(r.energy - ref["energy"]) < ref["tolerance"]
    assert abs(r.energy - ref["energy"]) < 5e-9
    # the last build's J and K against the oracle on the converged spin densities
    Ca, Cb = r.Ca[:, :ref["nalpha"]], r.Cb[:, :ref["nbeta"]]
    jko = dfjk_ref.OracleJK(df.to_pQq(), df.sparsity, df.nbf, df.naux)
    for jkx in (jk, jko):
        jkx.C_clear()
        jkx.C_left_add(np.ascontiguousarray(Ca))
        jkx.C_left_add(np.ascontiguousarray(Cb))
        jkx.compute()
    for a, b in zip(jk.J() + jk.K(), jko.J() + jko.K()):
        assert np.abs(np.asarray(a) - np.asarray(b)).max() < 1e-10
