"""Parity at the full configurations on real integrals: (H2O)_32 cc-pVTZ (nbf 1856, naux 4448,
nocc 160) and (H2O)_64 cc-pVDZ (nbf 1536, naux 7424, nocc 320).

B = J^-1/2 (P|mn) is built on the device from the engine's integral kernels
(psi4_gb300.device_init), exactly as the SCF workloads build it.  Orbitals are physical: the
core guess and an iterate four SCF iterations in.  Bars, all absolute (the parity bar: J and K
to 1e-10 in max absolute element against FP64):

* emulated-FP64 J/K against native FP64 J/K of the same engine: 1e-10;
* native FP64 J/K against the oracle's loop restatement of DFHelper (compute_J_symm /
  compute_K, dfhelper.cc:3162-3377) at the full nbf on a slice of 128 aux rows of the same B
  (the oracle cannot hold the whole tensor in its pQq layout in seconds): 1e-10;
* the precision form's K (BF16x3, FP32 accumulation) against native FP64: 1e-4 of max|K|.
  The split drops lo*lo and rounds lo to BF16 (about 2^-17 of each product), and the tensor
  cores' FP32 accumulation rounds toward zero over runs of up to 8192 terms (a bias of up
  to ~4096 ulp of a same-sign run, 2.4e-4 relative; cancellation keeps it well below that:
  4.9e-5 measured at (H2O)_32 cc-pVTZ on the core guess).  Its J is the FP64 J;
* the precision-form SCF (split-BF16 increments, emulated-FP64 anchor and final builds)
  converges to within 1 uEh of the emulated-FP64 SCF energy, with every iteration's energy
  error against FP64 at the same orbitals recorded and finite.
"""
import numpy as np
import pytest

from oracle import dfjk_ref
from psi4_gb300 import _jkabi as abi
from psi4_gb300.basis import BasisSet
from psi4_gb300.device_init import build_device_B, slice_pqq
from psi4_gb300.jk import DFJKEngine, GpuDFJK
from psi4_gb300.molecule import water_cluster
from psi4_gb300.scf import PrecisionSchedule, core_hamiltonian, energy_errors_vs_fp64, orthogonalizer, rhf

pytestmark = pytest.mark.gpu

CONFIGS = {"c2": ((4, 4, 2), "cc-pvtz"), "c3": ((4, 4, 4), "cc-pvdz")}
NQ_SLICE = 128
ABS_BAR = 1e-10


@pytest.fixture(scope="module", params=sorted(CONFIGS))
def real(request, ints_built, jk_built):
    lattice, basis = CONFIGS[request.param]
    mol = water_cluster(*lattice, seed=0)
    pb = BasisSet.build(mol, basis)
    ab = BasisSet.fitting_for(mol, pb)
    dd = build_device_B(mol, pb, ab, keep_rows=NQ_SLICE)
    ints = dd.ints
    H, S = core_hamiltonian(ints), ints.overlap()
    nocc = mol.nelectron // 2
    X = orthogonalizer(S)
    _, Cp = np.linalg.eigh(X.T @ H @ X)
    C_core = np.ascontiguousarray((X @ Cp)[:, :nocc])
    jk = GpuDFJK.from_engine(dd.engine)
    jk.set_precision("fp64-emulated")
    res = rhf(jk, H, S, nocc, mol.nuclear_repulsion_energy(), maxiter=4, fail_on_maxiter=False)
    C_mid = np.ascontiguousarray(res.C[:, :nocc])
    out = {"name": request.param, "mol": mol, "dd": dd, "H": H, "S": S, "nocc": nocc,
           "orbitals": {"core guess": C_core, "iteration 4": C_mid}}
    yield out
    dd.engine.close()


def _jk(eng, C, mode):
    J, K, _ = eng.compute(C, mode=mode)
    return J, K


def test_emulated_matches_native_fp64_absolute(real):
    eng = real["dd"].engine
    for label, C in real["orbitals"].items():
        Jn, Kn = _jk(eng, C, abi.DO_J | abi.DO_K)
        Je, Ke = _jk(eng, C, abi.DO_J | abi.DO_K | abi.EMULATED)
        dJ, dK = np.abs(Je - Jn).max(), np.abs(Ke - Kn).max()
        print(f"{real['name']} {label}: max|J| {np.abs(Jn).max():.3g} max|dJ| {dJ:.2e}  "
              f"max|K| {np.abs(Kn).max():.3g} max|dK| {dK:.2e}")
        assert dJ < ABS_BAR, (label, dJ)
        assert dK < ABS_BAR, (label, dK)


def test_mixed_k_against_native_fp64(real):
    eng = real["dd"].engine
    for label, C in real["orbitals"].items():
        Jn, Kn = _jk(eng, C, abi.DO_J | abi.DO_K)
        Jm, Km = _jk(eng, C, abi.DO_J | abi.DO_K | abi.MIXED)
        assert np.abs(Jm - Jn).max() < ABS_BAR
        rel = np.abs(Km - Kn).max() / np.abs(Kn).max()
        print(f"{real['name']} {label}: precision-form K relative error {rel:.2e}")
        assert rel < 1e-4, (label, rel)


def test_native_fp64_matches_oracle_on_an_aux_slice(real):
    dd = real["dd"]
    rows = dd.rows
    assert rows.shape[0] == NQ_SLICE
    eng = DFJKEngine(dd.nbf, NQ_SLICE, dd.sparsity.pair_mask)
    eng.upload_qtri(rows)
    Ppq, sp = slice_pqq(rows, dd.sparsity)
    tables = dfjk_ref.RowTables(sp, dd.nbf)
    try:
        for label, C in real["orbitals"].items():
            D = dfjk_ref.compute_D(C)
            Jo = dfjk_ref.compute_J_symm(Ppq, sp, D, dd.nbf, NQ_SLICE, tables)
            Ko = dfjk_ref.compute_K(Ppq, sp, C, C, dd.nbf, NQ_SLICE, True, tables)
            for form, mode in (("native", abi.DO_J | abi.DO_K), ("emulated", abi.DO_J | abi.DO_K | abi.EMULATED)):
                J, K = _jk(eng, C, mode)
                dJ, dK = np.abs(J - Jo).max(), np.abs(K - Ko).max()
                print(f"{real['name']} {label} {form} vs oracle ({NQ_SLICE} aux rows): max|dJ| {dJ:.2e} max|dK| {dK:.2e}")
                assert dJ < ABS_BAR and dK < ABS_BAR, (label, form, dJ, dK)
    finally:
        eng.close()


def test_precision_form_scf_within_one_microhartree(real):
    dd, mol = real["dd"], real["mol"]
    H, S, nocc = real["H"], real["S"], real["nocc"]
    e_nuc = mol.nuclear_repulsion_energy()
    jk = GpuDFJK.from_engine(dd.engine)
    jk.set_precision("fp64-emulated")
    ref = rhf(jk, H, S, nocc, e_nuc)
    jk.reset_incremental()
    sched = PrecisionSchedule(fp64_precision="fp64-emulated")
    res = rhf(jk, H, S, nocc, e_nuc, schedule=sched, record_orbitals=True)
    jk.set_incremental(False)
    jk.set_precision("fp64-emulated")
    errs = energy_errors_vs_fp64(res, jk, H, e_nuc)
    print(f"{real['name']}: FP64 {ref.energy:.10f} ({ref.iterations} it), precision form {res.energy:.10f} "
          f"({sched.n_mixed} mixed + {sched.n_fp64} FP64 builds), |dE| {abs(res.energy - ref.energy):.2e}; "
          f"per-iteration errors {[f'{e:.1e}' for e in errs]}")
    assert np.all(np.isfinite(errs))
    assert abs(res.energy - ref.energy) < 1e-6
    assert sched.n_mixed > 0 and sched.n_fp64 >= 2


def test_screened_device_build_matches_the_host_tensor(ints_built, jk_built):
    """build_device_B_screened (significant pairs only on the device, expanded back in blocks of
    aux rows for the block upload, as the C100H202 workload is built) gives the J and K of the
    host-built DF tensor, on a screened system with uneven upload blocks."""
    from psi4_gb300.device_init import build_device_B_screened
    from tests.helpers import system

    mol, pb, ab, ints, df = system("h2o_2_far", "cc-pvdz", 1e-5)
    assert 0.0 < df.sparsity.sparsity < 1.0
    dd = build_device_B_screened(mol, pb, ab, cutoff=1e-5, ints=ints, block=37, upload_rows=50)
    ref = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    ref.upload_qtri(df.B_tri)
    C = np.linalg.qr(np.random.default_rng(8).standard_normal((df.nbf, 10)))[0] * 0.5
    for mode in (abi.DO_J | abi.DO_K, abi.DO_J | abi.DO_K | abi.EMULATED):
        J, K = _jk(dd.engine, C, mode)
        Jr, Kr = _jk(ref, C, mode)
        assert np.abs(J - Jr).max() < ABS_BAR and np.abs(K - Kr).max() < ABS_BAR
    assert dd.timings["significant_pairs"] < dd.timings["pairs"]
    dd.engine.close()
    ref.close()
