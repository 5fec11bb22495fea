"""The differentiation form: torch.autograd over the engine's hand-written backward, and the
analytic DF-RHF nuclear gradient against central finite differences of the SCF energy
(step 0.005 bohr, 6 seeded coordinates — psi4's findif step, tests/fd-gradient/input.dat)."""
import numpy as np
import pytest

from oracle.backward_ref import jk_backward_dense
from psi4_gb300.jk import DFJKEngine
from tests.helpers import random_orbitals, system

pytestmark = pytest.mark.gpu


def test_autograd_matches_oracle(ints_built, jk_built):
    torch = pytest.importorskip("torch")
    from psi4_gb300.autograd import DFJK

    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz")
    eng = DFJKEngine(df.nbf, df.naux, None)
    eng.upload_qtri(df.B_tri)
    rng = np.random.default_rng(2)
    Cn = random_orbitals(df.nbf, 10, 3)
    wJ = rng.standard_normal((df.nbf, df.nbf))
    wK = rng.standard_normal((df.nbf, df.nbf))
    C = torch.tensor(Cn, device="cuda", requires_grad=True)
    B = torch.tensor(df.B_tri, device="cuda", requires_grad=True)
    J, K = DFJK.apply(C, B, eng)
    E = (torch.tensor(wJ, device="cuda") * J).sum() + (torch.tensor(wK, device="cuda") * K).sum()
    dC, dB = torch.autograd.grad(E, (C, B))
    dCr, dBr = jk_backward_dense(df.dense(), Cn, wJ, wK)
    assert np.abs(dC.cpu().numpy() - dCr).max() < 1e-10 * max(1, np.abs(dCr).max())
    assert np.abs(dB.cpu().numpy() - dBr).max() < 1e-10 * max(1, np.abs(dBr).max())


def _scf_energy_and_gradient(mol, want_grad):
    from psi4_gb300.basis import BasisSet
    from psi4_gb300.dfhelper import build_df_tensor
    from psi4_gb300.grad import rhf_gradient
    from psi4_gb300.ints import Integrals
    from psi4_gb300.jk import GpuDFJK
    from psi4_gb300.scf import core_hamiltonian, rhf

    pb = BasisSet.build(mol, "cc-pvdz")
    ab = BasisSet.fitting_for(mol, pb)
    ints = Integrals(mol, pb, ab)
    df = build_df_tensor(mol, pb, ab, ints=ints)
    jk = GpuDFJK.from_tensor(df)
    jk.initialize()
    res = rhf(jk, core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy(),
              e_conv=1e-12, d_conv=1e-10)
    g = None
    if want_grad:
        C = res.C[:, : res.nocc]
        D = C @ C.T
        _, Gamma = jk.engine.backward(C, 2.0 * D, -D, want_dC=False)
        g = rhf_gradient(mol, ints, df, res, Gamma, engine=jk.engine)  # M^-1/2 Gamma on the tensor cores
        g_host = rhf_gradient(mol, ints, df, res, Gamma)  # the same product in FP64 on the host
        # the digit product's error is relative to the row and column maxima of each run of 1024
        # aux functions (~1e-13 of them, against FP64's 1e-16 of each element); contracted with
        # the derivative integrals it moves the gradient by up to ~3e-8 Eh/bohr ((H2O)_16),
        # 30x below the differentiation form's 1e-6 bar
        assert np.abs(g - g_host).max() < 1e-7
    jk.finalize()
    return res.energy, g


def test_gradient_against_central_differences(ints_built, jk_built):
    mol, *_ = system("h2o_2", "cc-pvdz")
    E0, g = _scf_energy_and_gradient(mol, True)
    assert np.abs(g.sum(0)).max() < 1e-8  # translational invariance
    rng = np.random.default_rng(2024)
    h = 0.005
    picks = [(int(rng.integers(mol.natom)), int(rng.integers(3))) for _ in range(6)]
    for atom, axis in picks:
        Ep, _ = _scf_energy_and_gradient(mol.displaced(atom, axis, h), False)
        Em, _ = _scf_energy_and_gradient(mol.displaced(atom, axis, -h), False)
        fd = (Ep - Em) / (2 * h)
        print(f"atom {atom} axis {axis}: analytic {g[atom, axis]: .10f} fd {fd: .10f} diff {g[atom, axis] - fd: .2e}")
        assert abs(g[atom, axis] - fd) < 1e-5


def test_h2o16_gradient_against_central_differences(ints_built, jk_built):
    """The differentiation-form workload: (H2O)_16 (4x2x2 lattice, seed 0) cc-pVDZ /
    cc-pVDZ-jkfit, analytic gradient from the GPU backward vs central differences
    (0.005 bohr) on 6 seeded coordinates."""
    from psi4_gb300.molecule import water_cluster

    mol = water_cluster(4, 2, 2, seed=0)
    E0, g = _scf_energy_and_gradient(mol, True)
    assert np.abs(g.sum(0)).max() < 1e-7
    rng = np.random.default_rng(16)
    h = 0.005
    worst = 0.0
    for _ in range(6):
        atom, axis = int(rng.integers(mol.natom)), int(rng.integers(3))
        Ep, _ = _scf_energy_and_gradient(mol.displaced(atom, axis, h), False)
        Em, _ = _scf_energy_and_gradient(mol.displaced(atom, axis, -h), False)
        fd = (Ep - Em) / (2 * h)
        worst = max(worst, abs(g[atom, axis] - fd))
        print(f"(H2O)_16 atom {atom} axis {axis}: analytic {g[atom, axis]: .9f} fd {fd: .9f} diff {g[atom, axis] - fd: .2e}")
    assert worst < 1e-6  # the differentiation form's bar (Eh/bohr)
