"""The gradient path for systems whose dense 3-index arrays do not fit (C100H202): Gamma from
the engine's aux-batched backward (gdfjk_backward_gamma_device, (Q|mi) recomputed per batch,
Y = gK X on the tensor cores) in the significant-pair layout, then the metric products, the
Frechet derivative and the derivative contractions on the device.

Bars: Gamma against gdfjk_backward's all-FP64 Gamma, 1e-11 of max|Gamma| (the digit product's
error is relative to the row and column maxima); the whole two-electron gradient against the
dense device path, 1e-7 Eh/bohr (W = Gamma A^T as a digit product, as measured at (H2O)_16:
5e-8), both far below the differentiation form's 1e-6."""
import numpy as np
import pytest

from tests.helpers import system

pytestmark = pytest.mark.gpu
torch = pytest.importorskip("torch")
DEV = torch.device("cuda:0")


def _scf(dd, ints, mol):
    from psi4_gb300.jk import GpuDFJK
    from psi4_gb300.scf import core_hamiltonian, rhf

    jk = GpuDFJK.from_engine(dd.engine)
    res = rhf(jk, core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy(),
              e_conv=1e-10, d_conv=1e-8)
    return res


@pytest.fixture(scope="module")
def h2o8():
    from psi4_gb300.device_init import build_device_B_screened

    mol, pb, ab, ints, df = system("h2o_8", "cc-pvdz")
    dd = build_device_B_screened(mol, pb, ab, ints=ints)
    res = _scf(dd, ints, mol)
    return mol, ints, df, dd, res


@pytest.mark.parametrize("batch_q", [97, 0])
def test_backward_gamma_matches_full_backward(ints_built, jk_built, h2o8, batch_q):
    mol, ints, df, dd, res = h2o8
    eng = dd.engine
    C = res.C[:, :res.nocc].copy()
    D = C @ C.T
    _, Gref = eng.backward(C, 2.0 * D, -D, want_dC=False)
    nbf, nocc = C.shape
    npair = nbf * (nbf + 1) // 2
    Cd = torch.from_numpy(C).to(DEV)
    Dd = Cd @ Cd.T
    gJ, gK = 2.0 * Dd, -Dd
    G = torch.empty((dd.naux, npair), dtype=torch.float64, device=DEV)
    eng.backward_gamma_device(Cd.data_ptr(), nocc, nocc, gJ.data_ptr(), gK.data_ptr(), G.data_ptr(), npair,
                              batch_q=batch_q)
    d = np.abs(G.cpu().numpy() - Gref).max()
    print(f"batch {batch_q}: max|Gamma| {np.abs(Gref).max():.3e} max|d| {d:.2e}")
    assert d <= 1e-11 * np.abs(Gref).max()
    # the significant-pair layout through a column map
    r, c = np.tril_indices(nbf)
    sig = np.flatnonzero(dd.sparsity.pair_mask[r, c])
    col_map = np.full(npair, -1, dtype=np.int64)
    col_map[sig] = np.arange(sig.size)
    col_d = torch.from_numpy(col_map).to(DEV)
    Gs = torch.empty((dd.naux, sig.size), dtype=torch.float64, device=DEV)
    eng.backward_gamma_device(Cd.data_ptr(), nocc, nocc, gJ.data_ptr(), gK.data_ptr(), Gs.data_ptr(), sig.size,
                              col_map_ptr=col_d.data_ptr(), batch_q=batch_q)
    assert np.abs(Gs.cpu().numpy() - Gref[:, sig]).max() <= 1e-11 * np.abs(Gref).max()


def test_screened_gradient_matches_dense_device_path(ints_built, jk_built, h2o8):
    from psi4_gb300.grad import two_electron_gradient, two_electron_gradient_screened

    mol, ints, df, dd, res = h2o8
    C = res.C[:, :res.nocc].copy()
    D = C @ C.T
    _, Gamma = dd.engine.backward(C, 2.0 * D, -D, want_dC=False)
    g_dense = two_electron_gradient(ints, dd, Gamma, engine=dd.engine)
    tm = {}
    g_scr = two_electron_gradient_screened(dd.engine, ints, dd.sparsity, dd.metric, dd.Jmhalf, C, timings=tm,
                                           batch_q=150)
    d = np.abs(g_scr - g_dense).max()
    print(f"(H2O)_8 screened vs dense two-electron gradient: max|g| {np.abs(g_dense).max():.3e} max|d| {d:.2e}; {tm}")
    assert d < 1e-7
    assert np.abs(g_scr.sum(0)).max() < 1e-8
