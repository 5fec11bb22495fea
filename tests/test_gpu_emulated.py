"""The emulated-FP64 form on the GPU: K from BF16 tensor-core products of 7-bit digit slices
(exact FP32 level sums, double-float epilogue) against the FP64 oracle.

The digits are fixed point relative to each row's (or row group's) largest element, so the
error scales with the magnitude of the operands rather than with each result element:
on physical (SCF) orbitals K meets the FP64 bar of 1e-10 max absolute; on random U(0,1)
orbitals, where |K| reaches 1e3-1e5, the bound is 1e-10 + 1e-11 max|K|."""
import os

import numpy as np
import pytest

from oracle import dfjk_ref
from psi4_gb300 import _jkabi as abi
from psi4_gb300.jk import DFJKEngine, GdfjkError, GpuDFJK
from tests.helpers import random_orbitals, reference_values, system

pytestmark = pytest.mark.gpu
TOL = 1e-10
EMU = abi.DO_J | abi.DO_K | abi.EMULATED


def _random_bound(Kref):
    """Bound for random, unnormalised orbitals: 1e-10 + 1e-11 max|K|.

    Why relative there: U(0,1) orbitals drive |X| and |K| to 1e3-1e5 (no physical density
    does that), and the digits are fixed point relative to each row's (or row group's)
    largest magnitude, so the emulation's error scales with max|K| (49-bit digits less the
    double-float accumulation: ~1e-11 relative at worst) rather than with each element, as
    FP64 rounding would.  On physical orbitals the absolute bar holds unchanged: see
    test_emulated_scf_orbitals_strict here and tests/test_gpu_realsize.py (7e-12 at
    (H2O)_32 cc-pVTZ and (H2O)_64 cc-pVDZ on real integrals)."""
    return TOL + 1e-11 * np.abs(Kref).max()


def _k_fp64(df, C):
    return dfjk_ref.compute_K(df.to_pQq(), df.sparsity, C, C, df.nbf, df.naux)


def _engine(df):
    eng = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    eng.upload_pqq(df.to_pQq(), df.sparsity)
    return eng


def _scf_orbitals(name, basis):
    from psi4_gb300.scf import core_hamiltonian, rhf

    mol, pb, ab, ints, df = system(name, basis)
    jko = dfjk_ref.OracleJK(df.to_pQq(), df.sparsity, df.nbf, df.naux)
    nocc = mol.nelectron // 2
    res = rhf(jko, core_hamiltonian(ints), ints.overlap(), nocc, mol.nuclear_repulsion_energy(), e_conv=1e-8,
              d_conv=1e-6)
    return df, res.C[:, :nocc].copy()


def test_emulated_scf_orbitals_strict(ints_built, jk_built):
    """(H2O)_8 cc-pVDZ converged orbitals: J and K within 1e-10 of the oracle."""
    df, C = _scf_orbitals("h2o_8", "cc-pvdz")
    eng = _engine(df)
    J, K, _ = eng.compute(C, mode=EMU)
    Jr, Kr = dfjk_ref.compute_J_symm(df.to_pQq(), df.sparsity, C @ C.T, df.nbf, df.naux), _k_fp64(df, C)
    print(f"emulated K on SCF orbitals: max|K| {np.abs(Kr).max():.3f} max|dK| {np.abs(K - Kr).max():.2e}")
    assert np.abs(J - Jr).max() < TOL
    assert np.abs(K - Kr).max() < TOL
    assert np.abs(K - K.T).max() == 0.0


@pytest.mark.parametrize("case", [("h2o", "cc-pvdz", 1e-12), ("h2o_2", "cc-pvdz", 1e-12), ("h2o", "cc-pvtz", 1e-12),
                                  ("h2o_2_far", "cc-pvdz", 1e-5)])
@pytest.mark.parametrize("nocc", [5, 40, 70, 200])
def test_emulated_random_orbitals(ints_built, jk_built, case, nocc):
    mol, pb, ab, ints, df = system(*case)
    eng = _engine(df)
    C = random_orbitals(df.nbf, nocc, seed=nocc) * 0.3
    _, K, _ = eng.compute(C, mode=EMU)
    Kr = _k_fp64(df, C)
    err = np.abs(K - Kr).max()
    print(f"{case[0]}/{case[1]} nocc {nocc}: max|K| {np.abs(Kr).max():.3e} max|dK| {err:.2e}")
    assert err < _random_bound(Kr)


def test_emulated_determinism_and_batches(ints_built, jk_built, monkeypatch):
    """Repeated builds are bitwise identical; cutting the aux range into many batches (tiny X
    buffer cap) gives the same K to rounding."""
    df, C = _scf_orbitals("h2o_8", "cc-pvdz")
    eng = _engine(df)
    _, K1, _ = eng.compute(C, mode=EMU)
    _, K2, _ = eng.compute(C, mode=EMU)
    assert np.array_equal(K1, K2)
    monkeypatch.setenv("GDFJK_OZ_XCAP_GB", "0.002")
    eng2 = _engine(df)
    _, K3, _ = eng2.compute(C, mode=EMU)
    Kr = _k_fp64(df, C)
    print(f"batched: max|dK| {np.abs(K3 - Kr).max():.2e}, vs one batch {np.abs(K3 - K1).max():.2e}")
    assert np.abs(K3 - Kr).max() < TOL
    assert np.abs(K3 - K1).max() < 1e-12


def test_emulated_long_k_runs(jk_built):
    """nbf 2100 (2176 padded, over the 2048 terms of one run): the half-transform's k range is
    cut into two accumulation runs, the second added to the first in double-float.
    Synthetic B on the device; reference: plain torch FP64."""
    torch = pytest.importorskip("torch")
    nbf, naux, nocc = 2100, 16, 96
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev)
    g.manual_seed(7)
    npair = nbf * (nbf + 1) // 2
    Bt = torch.randn((naux, npair), dtype=torch.float64, device=dev, generator=g) * 0.02
    eng = DFJKEngine(nbf, naux, None)
    eng.upload_device(Bt.data_ptr())
    rows, cols = torch.tril_indices(nbf, nbf, device=dev)
    Bd = torch.zeros((naux, nbf, nbf), dtype=torch.float64, device=dev)
    Bd[:, rows, cols] = Bt
    Bd[:, cols, rows] = Bt
    C = torch.randn((nbf, nocc), dtype=torch.float64, device=dev, generator=g) * 0.1
    X = torch.matmul(Bd, C)  # naux x nbf x nocc
    Kr = torch.einsum("qmi,qni->mn", X, X).cpu().numpy()
    del Bd, X
    _, K, _ = eng.compute(C.cpu().numpy(), mode=abi.DO_K | abi.EMULATED)
    err = np.abs(K - Kr).max()
    print(f"nbf {nbf}: max|K| {np.abs(Kr).max():.3e} max|dK| {err:.2e}")
    assert err < _random_bound(Kr)


def test_emulated_scf2_energy(ints_built, jk_built):
    """GpuDFJK with precision fp64-emulated reproduces the scf2 reference energy (1e-9)."""
    from psi4_gb300.scf import core_hamiltonian, rhf

    ref = reference_values()["scf2"]
    mol, pb, ab, ints, df = system("h2o_scf2", "cc-pvtz")
    jk = GpuDFJK.from_tensor(df)
    jk.set_precision("fp64-emulated")
    jk.initialize()
    r = rhf(jk, core_hamiltonian(ints), ints.overlap(), mol.nelectron // 2, mol.nuclear_repulsion_energy(),
            e_conv=1e-10, d_conv=1e-8)
    print(f"scf2 emulated: {r.energy:.12f} ref {ref['energy']:.12f}")
    assert abs(r.energy - ref["energy"]) < ref["tolerance"]


def test_emulated_anchor_in_precision_schedule(ints_built, jk_built):
    """The precision form with emulated FP64 anchors and final builds converges to the FP64
    SCF energy."""
    from psi4_gb300.scf import PrecisionSchedule, core_hamiltonian, rhf

    mol, pb, ab, ints, df = system("h2o_8", "cc-pvdz")
    args = (core_hamiltonian(ints), ints.overlap(), 40, mol.nuclear_repulsion_energy())
    jk64 = GpuDFJK.from_tensor(df)
    jk64.initialize()
    e64 = rhf(jk64, *args, e_conv=1e-10, d_conv=1e-8).energy
    jk = GpuDFJK.from_tensor(df)
    jk.initialize()
    r = rhf(jk, *args, e_conv=1e-10, d_conv=1e-8, schedule=PrecisionSchedule(fp64_precision="fp64-emulated"))
    print(f"schedule with emulated FP64 builds: {r.energy:.12f} vs FP64 {e64:.12f}")
    assert abs(r.energy - e64) < 1e-9


def test_emulated_block_sparse(jk_built):
    """A banded pair mask (nbf 640: 10 x 10 tiles, about a third stored): the int8 digits of B
    are kept only for the 128 x 32 blocks that touch a stored tile, and the half-transform
    walks only those.  Compared with the native FP64 K of the same engine; `trim` releases the
    digit copy, which is rebuilt identically."""
    torch = pytest.importorskip("torch")
    nbf, naux, nocc = 640, 96, 40
    idx = np.arange(nbf)
    mask = (np.abs(idx[:, None] - idx[None, :]) < 90).astype(np.uint8)
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    r, c = np.tril_indices(nbf)
    tri = torch.from_numpy(mask[r, c].astype(np.float64)).to(dev)
    Bt = torch.randn((naux, tri.numel()), dtype=torch.float64, device=dev, generator=g) * 0.05 * tri
    eng = DFJKEngine(nbf, naux, mask)
    eng.upload_device_block(Bt.data_ptr(), 0, naux // 2)
    eng.upload_device_block(Bt[naux // 2:].data_ptr(), naux // 2, naux - naux // 2)
    C = np.random.default_rng(4).standard_normal((nbf, nocc)) * 0.2
    _, K64, _ = eng.compute(C, mode=abi.DO_K)
    _, Ke, _ = eng.compute(C, mode=abi.DO_K | abi.EMULATED)
    err = np.abs(Ke - K64).max()
    print(f"block-sparse emulated K: max|K| {np.abs(K64).max():.3e} max|dK| {err:.2e}")
    assert err < _random_bound(K64)
    eng.trim()
    _, Ke2, _ = eng.compute(C, mode=abi.DO_K | abi.EMULATED)
    assert np.array_equal(Ke, Ke2)


@pytest.mark.parametrize("case", [("h2o", "cc-pvdz"), ("h2o_2", "cc-pvdz"), ("h2o_2_far", "cc-pvdz")])
@pytest.mark.parametrize("nocc", [16, 20, 30])
def test_emulated_nonsymmetric_pairs(ints_built, jk_built, case, nocc):
    """tests/pytests/test_dfjk.py style random C_left != C_right pairs: K = sum_Q (B_Q Cl)(B_Q Cr)^T
    from two half-transforms and a contraction over every tile; J is native FP64."""
    mol, pb, ab, ints, df = system(*case)
    eng = _engine(df)
    Cl = random_orbitals(df.nbf, nocc, seed=100 + nocc)
    Cr = random_orbitals(df.nbf, nocc, seed=200 + nocc)
    J, K, _ = eng.compute(Cl, Cr, mode=EMU)
    J64, K64, _ = eng.compute(Cl, Cr, mode=abi.DO_J | abi.DO_K)
    Kr = dfjk_ref.compute_K(df.to_pQq(), df.sparsity, Cl, Cr, df.nbf, df.naux, lr_symmetric=False)
    err = np.abs(K - Kr).max()
    print(f"{case[0]} nocc {nocc}: max|K| {np.abs(Kr).max():.3e} max|dK| {err:.2e} (native {np.abs(K64 - Kr).max():.2e})")
    assert np.array_equal(J, J64)
    assert err < _random_bound(Kr)
    assert np.abs(K - K.T).max() > 0  # really non-symmetric


def test_emulated_nonsymmetric_batches_and_jk_front_end(ints_built, jk_built, monkeypatch):
    """Many aux batches (K accumulated over them in place) and GpuDFJK's C_left/C_right pairs
    routed to the emulated form."""
    df, C = _scf_orbitals("h2o_8", "cc-pvdz")
    Cr = C + 0.01 * random_orbitals(df.nbf, C.shape[1], seed=5)
    Kr = dfjk_ref.compute_K(df.to_pQq(), df.sparsity, C, Cr, df.nbf, df.naux, lr_symmetric=False)
    monkeypatch.setenv("GDFJK_OZ_XCAP_GB", "0.002")
    _, K, _ = _engine(df).compute(C, Cr, mode=EMU)
    assert np.abs(K - Kr).max() < TOL
    monkeypatch.delenv("GDFJK_OZ_XCAP_GB")
    jk = GpuDFJK.from_tensor(df)
    jk.set_precision("fp64-emulated")
    jk.initialize()
    jk.C_left_add(C)
    jk.C_right_add(Cr)
    jk.compute()
    assert np.abs(jk.K()[0] - Kr).max() < TOL


def test_emulated_rejects_wide_occupation(jk_built):
    """More than 1024 occupied columns would overrun one exact contraction run: refused with a
    clear error (GpuDFJK routes such densities to the native FP64 K)."""
    nbf, naux = 128, 8
    eng = DFJKEngine(nbf, naux, None)
    rng = np.random.default_rng(1)
    r, c = np.tril_indices(nbf)
    eng.upload_qtri(rng.standard_normal((naux, r.size)) * 0.01)
    C = rng.standard_normal((nbf, 1040)) * 0.01
    with pytest.raises(GdfjkError, match="nocc above 1024"):
        eng.compute(C, mode=abi.DO_K | abi.EMULATED)
    _, K, _ = eng.compute(C, mode=abi.DO_K)  # the engine stays usable
    assert np.isfinite(K).all()


@pytest.mark.parametrize("nocc", [401, 702])
def test_emulated_wide_factors(ints_built, jk_built, nocc):
    """Factors wider than the basis (as the SAD guess's natural orbitals of a large molecule
    are: 702 columns for C100H202): the emulated K against native FP64 with one aux function
    per contraction group (nocc_pad 704) or two (416)."""
    mol, pb, ab, ints, df = system("h2o_8")
    eng = _engine(df)
    C = np.random.default_rng(nocc).standard_normal((df.nbf, nocc)) * 0.05
    _, Kn, _ = eng.compute(C, mode=abi.DO_J | abi.DO_K)
    _, Ke, _ = eng.compute(C, mode=EMU)
    err = np.abs(Ke - Kn).max()
    print(f"nocc {nocc}: max|K| {np.abs(Kn).max():.3e} max|dK| {err:.2e}")
    assert err < _random_bound(Kn)
    eng.close()


def test_emulated_batch_buffers_follow_the_column_count(ints_built, jk_built, monkeypatch):
    """A build with more occupied columns after one with fewer, on one engine, where the second
    gets a smaller aux batch (qb 5 against 8) that still needs larger X buffers (5 x 704 > 8 x
    416 column pairs): the buffers grow, and both builds agree with native FP64."""
    mol, pb, ab, ints, df = system("h2o_8")
    eng = _engine(df)
    monkeypatch.setenv("GDFJK_OZ_XCAP_GB", "0.02")
    for nocc in (401, 702):
        C = np.random.default_rng(nocc + 1).standard_normal((df.nbf, nocc)) * 0.05
        _, Kn, _ = eng.compute(C, mode=abi.DO_J | abi.DO_K)
        _, Ke, _ = eng.compute(C, mode=EMU)
        assert np.abs(Ke - Kn).max() < _random_bound(Kn)
    eng.close()
