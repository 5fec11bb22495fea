"""GPU reverse mode (gdfjk_backward) against the oracle, and the RHF nuclear gradient with the
GPU Gamma against the reference's scf6 values and central finite differences."""
import numpy as np
import pytest

from oracle.backward_ref import jk_backward_dense
from psi4_gb300.jk import DFJKEngine
from tests.helpers import random_orbitals, reference_values, system

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [("h2o", "cc-pvdz", 1e-12), ("h2o_2", "cc-pvdz", 1e-12), ("h2o_2_far", "cc-pvdz", 1e-5)])
def test_backward_matches_oracle(ints_built, jk_built, case):
    mol, pb, ab, ints, df = system(*case)
    eng = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    eng.upload_pqq(df.to_pQq(), df.sparsity)
    rng = np.random.default_rng(11)
    C = random_orbitals(df.nbf, 7, 12)
    gJ = rng.standard_normal((df.nbf, df.nbf))
    gK = rng.standard_normal((df.nbf, df.nbf))
    dC, G = eng.backward(C, gJ, gK)
    dCr, Gr = jk_backward_dense(df.dense(), C, gJ, gK)
    assert np.abs(dC - dCr).max() < 1e-10 * max(1.0, np.abs(dCr).max())
    # Gamma is compared on the stored (significant) tiles; the oracle covers every pair
    assert np.abs(G - Gr).max() < 1e-10 * max(1.0, np.abs(Gr).max())


def test_rhf_gradient_on_gpu_scf6(ints_built, jk_built):
    from psi4_gb300.grad import rhf_gradient
    from psi4_gb300.jk import GpuDFJK
    from psi4_gb300.scf import core_hamiltonian, rhf

    ref = reference_values()["scf6_rhf_gradient"]
    mol, pb, ab, ints, df = system("h2o_c2v", "cc-pvdz")
    jk = GpuDFJK.from_tensor(df)
    jk.initialize()
    res = rhf(jk, core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy(),
              e_conv=1e-10, d_conv=1e-10)
    C = res.C[:, : res.nocc]
    D = C @ C.T
    _, Gamma = jk.engine.backward(C, 2.0 * D, -D, want_dC=False)
    g = rhf_gradient(mol, ints, df, res, Gamma)
    assert np.abs(g - np.array(ref["gradient"])).max() < ref["tolerance"]
