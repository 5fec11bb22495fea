"""The precision form on the GPU: split-BF16 tensor-core K (tcgen05) against FP64, full and
incremental builds, and the precision-form SCF against the FP64 SCF energy."""
import numpy as np
import pytest

from oracle import dfjk_ref
from psi4_gb300 import _jkabi as abi
from psi4_gb300.jk import DFJKEngine, GpuDFJK, density_difference_factor
from tests.helpers import random_orbitals, system

pytestmark = pytest.mark.gpu
# BF16x3 (hi*hi + hi*lo + lo*hi, FP32 accumulation): ~2^-16 relative per product
REL_TOL = 2e-4


def _k_fp64(df, C):
    return dfjk_ref.compute_K(df.to_pQq(), df.sparsity, C, C, df.nbf, df.naux)


@pytest.fixture(scope="module")
def h2o8(ints_built, jk_built):
    mol, pb, ab, ints, df = system("h2o_8", "cc-pvdz")
    eng = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    eng.upload_pqq(df.to_pQq(), df.sparsity)
    return mol, ints, df, eng


@pytest.mark.parametrize("case", [("h2o", "cc-pvdz", 1e-12), ("h2o_2", "cc-pvdz", 1e-12), ("h2o", "cc-pvtz", 1e-12)])
@pytest.mark.parametrize("nocc", [5, 40, 70])
def test_mixed_full_build_small(ints_built, jk_built, case, nocc):
    mol, pb, ab, ints, df = system(*case)
    eng = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    eng.upload_pqq(df.to_pQq(), df.sparsity)
    C = random_orbitals(df.nbf, nocc, seed=nocc) * 0.3
    J, K, _ = eng.compute(C, mode=abi.DO_J | abi.DO_K | abi.MIXED)
    Kr = _k_fp64(df, C)
    Jr = dfjk_ref.compute_J_symm(df.to_pQq(), df.sparsity, C @ C.T, df.nbf, df.naux)
    err = np.abs(K - Kr).max() / np.abs(Kr).max()
    print(f"mixed K rel err {err:.3e}")
    assert err < REL_TOL
    assert np.abs(J - Jr).max() < 1e-10  # J stays FP64
    assert np.abs(K - K.T).max() == 0.0


def test_mixed_h2o8_and_determinism(h2o8):
    mol, ints, df, eng = h2o8
    C = random_orbitals(df.nbf, 40, seed=5) * 0.2
    _, K1, _ = eng.compute(C, mode=abi.DO_K | abi.MIXED)
    _, K2, _ = eng.compute(C, mode=abi.DO_K | abi.MIXED)
    assert np.array_equal(K1, K2)
    Kr = _k_fp64(df, C)
    assert np.abs(K1 - Kr).max() / np.abs(Kr).max() < REL_TOL


def test_incremental_build(h2o8):
    mol, ints, df, eng = h2o8
    rng = np.random.default_rng(8)
    C1 = random_orbitals(df.nbf, 40, seed=6) * 0.2
    C2 = C1 + 0.01 * rng.standard_normal(C1.shape)
    J1, K1 = eng.compute_incremental(C1, C1, 40, reset=True)
    U, npos = density_difference_factor(C2, C1)
    assert 0 < npos < U.shape[1]  # both signs present
    J2, K2 = eng.compute_incremental(C2, U, npos)
    K1r, K2r = _k_fp64(df, C1), _k_fp64(df, C2)
    e1 = np.abs(K1 - K1r).max()
    e2 = np.abs(K2 - K2r).max()
    # the increment adds an error proportional to |dK|, far below the first build's
    de = np.abs((K2 - K1) - (K2r - K1r)).max()
    print(f"full {e1:.3e}  after increment {e2:.3e}  increment error {de:.3e}  |dK| {np.abs(K2r - K1r).max():.3e}")
    assert de < REL_TOL * np.abs(K2r - K1r).max() * 5
    assert e2 < e1 + de + 1e-12
    Jr = dfjk_ref.compute_J_symm(df.to_pQq(), df.sparsity, C2 @ C2.T, df.nbf, df.naux)
    assert np.abs(J2 - Jr).max() < 1e-10


def test_precision_form_scf_h2o8(h2o8):
    """(H2O)_8 cc-pVDZ: mixed incremental builds, then FP64 final rebuilds; the converged
    energy equals the FP64 SCF energy within 1 uEh (here much tighter)."""
    from psi4_gb300.scf import PrecisionSchedule, core_hamiltonian, rhf

    mol, ints, df, eng = h2o8
    H, S = core_hamiltonian(ints), ints.overlap()
    ref = GpuDFJK.from_tensor(df)
    ref.initialize()
    r64 = rhf(ref, H, S, 40, mol.nuclear_repulsion_energy())
    jk = GpuDFJK.from_tensor(df)
    jk.initialize()
    sched = PrecisionSchedule(report_fp64=ref)
    rmx = rhf(jk, H, S, 40, mol.nuclear_repulsion_energy(), schedule=sched)
    errs = [e.get("energy_error_vs_fp64") for e in rmx.log if "energy_error_vs_fp64" in e]
    print("fp64 iters", r64.iterations, "mixed", sched.n_mixed, "fp64 (incl. anchor)", sched.n_fp64, "anchor", sched.n_anchor,
          "max |E_mixed - E_fp64| per iteration", max(abs(x) for x in errs))
    assert rmx.converged
    assert abs(rmx.energy - r64.energy) < 1e-6
    assert abs(rmx.energy - r64.energy) < 1e-9
    assert sched.n_fp64 >= 2


def test_mixed_block_sparse(jk_built):
    """Banded pair mask (nbf 640): the split copy of B keeps only the 128 x 32 blocks that
    touch a stored tile; the mixed K matches the native FP64 K of the same engine to the
    BF16x3 tolerance, full and incremental."""
    torch = pytest.importorskip("torch")
    nbf, naux, nocc = 640, 96, 40
    idx = np.arange(nbf)
    mask = (np.abs(idx[:, None] - idx[None, :]) < 90).astype(np.uint8)
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev)
    g.manual_seed(12)
    r, c = np.tril_indices(nbf)
    tri = torch.from_numpy(mask[r, c].astype(np.float64)).to(dev)
    Bt = torch.randn((naux, tri.numel()), dtype=torch.float64, device=dev, generator=g) * 0.05 * tri
    eng = DFJKEngine(nbf, naux, mask)
    eng.upload_device_block(Bt.data_ptr(), 0, naux)
    C = np.random.default_rng(5).standard_normal((nbf, nocc)) * 0.2
    _, K64, _ = eng.compute(C, mode=abi.DO_K)
    _, Km, _ = eng.compute(C, mode=abi.DO_K | abi.MIXED)
    err = np.abs(Km - K64).max() / np.abs(K64).max()
    print(f"block-sparse mixed K rel err {err:.2e}")
    assert err < REL_TOL


def test_incremental_device_entry_matches_host_entry(ints_built, jk_built):
    """gdfjk_compute_incremental_device (device buffers, asynchronous) gives bitwise the host
    entry's J and K, for a full split build and an increment, and so does J enqueued on its
    own before the K increment (the order GpuDFJK uses to overlap the host's factor of dD)."""
    torch = pytest.importorskip("torch")
    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz")
    nbf = df.nbf
    C1 = np.linalg.qr(np.random.default_rng(31).standard_normal((nbf, 10)))[0] * 0.5
    C2 = C1 + 0.01 * np.random.default_rng(32).standard_normal((nbf, 10))
    U, npos = density_difference_factor(C2, C1)
    host = DFJKEngine(nbf, df.naux, None)
    host.upload_qtri(df.B_tri)
    host.compute_incremental(C1, C1, 10, reset=True)
    Jh, Kh = host.compute_incremental(C2, U, npos)
    dev = DFJKEngine(nbf, df.naux, None)
    dev.upload_qtri(df.B_tri)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()
    C1d, C2d, Ud = t(C1), t(C2), t(U)
    Jd = torch.empty((nbf, nbf), dtype=torch.float64, device="cuda")
    Kd = torch.empty_like(Jd)
    torch.cuda.synchronize()
    m = abi.DO_J | abi.DO_K | abi.MIXED
    dev.compute_incremental_device(C1d.data_ptr(), 10, 10, C1d.data_ptr(), 10, 10, 10, m | abi.RESET, Jd.data_ptr(),
                                   Kd.data_ptr())
    dev.compute_incremental_device(C2d.data_ptr(), 10, 10, None, 0, 0, 1, abi.DO_J, Jd.data_ptr(), None)
    dev.compute_incremental_device(C2d.data_ptr(), 10, 10, Ud.data_ptr(), U.shape[1], npos, U.shape[1],
                                   abi.DO_K | abi.MIXED, None, Kd.data_ptr())
    dev.synchronize()
    assert np.array_equal(Jd.cpu().numpy(), Jh) and np.array_equal(Kd.cpu().numpy(), Kh)
    host.close()
    dev.close()

