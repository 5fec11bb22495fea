"""Long-range exchange wK (range-separated functionals): wK = sum_Q (J^-1 (Q|mn) C_l)((Q|w|mn) C_r)^T
on the GPU (gdfjk_compute_wK: the two tensors in two engines; native FP64 and the emulated
form) against the oracle's restatement of DFHelper::compute_wK, and through GpuDFJK's
set_do_wK / set_omega / wK()."""
import numpy as np
import pytest

from oracle import dfjk_ref
from psi4_gb300 import _jkabi as abi
from psi4_gb300.dfhelper import build_wk_tensors
from psi4_gb300.jk import DFJKEngine, GdfjkError, GpuDFJK
from tests.helpers import random_orbitals, system

pytestmark = pytest.mark.gpu
OMEGA = 0.4


def _engines(df, m1, w):
    out = []
    for t in (m1, w):
        e = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
        e.upload_qtri(t.B_tri)
        out.append(e)
    return out


@pytest.mark.parametrize("case", [("h2o", "cc-pvdz"), ("h2o_2", "cc-pvdz"), ("h2o", "cc-pvtz")])
def test_wk_engine_against_oracle(ints_built, jk_built, case):
    mol, pb, ab, ints, df = system(*case)
    m1, w = build_wk_tensors(df, ints, OMEGA)
    left, right = _engines(df, m1, w)
    Cl = random_orbitals(df.nbf, 12, seed=3) * 0.3
    Cr = random_orbitals(df.nbf, 12, seed=4) * 0.3
    for lr in (True, False):
        ref = dfjk_ref.compute_wK(m1.to_pQq(), w.to_pQq(), df.sparsity, Cl, None if lr else Cr, df.nbf, df.naux,
                                  lr_symmetric=lr)
        for mode, tol in ((0, 1e-10), (abi.EMULATED, 1e-10 + 1e-11 * np.abs(ref).max())):
            got = left.compute_wK(right, Cl, None if lr else Cr, mode=mode)
            err = np.abs(got - ref).max()
            print(f"{case} lr={lr} mode={mode}: max|wK| {np.abs(ref).max():.3e} max|dwK| {err:.2e}")
            assert err < tol
            if lr:
                assert np.array_equal(got, got.T)


def test_wk_through_gpudfjk(ints_built, jk_built):
    """GpuDFJK with set_do_wK(True): J and K as before, wK from the two extra tensors
    (MemDFJK::compute_JK with do_wK, MemDFJK.cc:97-111), in native and emulated FP64."""
    mol, pb, ab, ints, df = system("h2o", "cc-pvdz")
    m1, w = build_wk_tensors(df, ints, OMEGA)
    C = random_orbitals(df.nbf, 5, seed=9) * 0.3
    ref = dfjk_ref.compute_wK(m1.to_pQq(), w.to_pQq(), df.sparsity, C, None, df.nbf, df.naux)
    for precision in ("fp64", "fp64-emulated"):
        jk = GpuDFJK.build(pb, ab, mol)
        jk.set_precision(precision)
        jk.set_do_wK(True)
        jk.set_omega(OMEGA)
        jk.initialize()
        jk.C_left_add(C)
        jk.compute()
        assert np.abs(jk.wK()[0] - ref).max() < 1e-10
        Kr = dfjk_ref.compute_K(df.to_pQq(), df.sparsity, C, C, df.nbf, df.naux)
        assert np.abs(jk.K()[0] - Kr).max() < 1e-10


def test_wk_rejects_mismatched_handles(jk_built):
    a = DFJKEngine(64, 16, None)
    b = DFJKEngine(64, 24, None)
    rng = np.random.default_rng(0)
    n = 64 * 65 // 2
    a.upload_qtri(rng.standard_normal((16, n)) * 0.01)
    b.upload_qtri(rng.standard_normal((24, n)) * 0.01)
    with pytest.raises(GdfjkError, match="must share"):
        a.compute_wK(b, rng.standard_normal((64, 4)))
