"""B uploaded in blocks of aux functions (gdfjk_upload_B_block / _device_block) gives the
same J and K, bit for bit, as the one-shot upload; blocks out of order are refused."""
import numpy as np
import pytest

from psi4_gb300 import _jkabi as abi
from psi4_gb300.jk import DFJKEngine, GdfjkError
from tests.helpers import random_orbitals, system

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [("h2o_2", "cc-pvdz", 1e-12), ("h2o_2_far", "cc-pvdz", 1e-5)])
def test_block_upload_matches_full(ints_built, jk_built, case):
    mol, pb, ab, ints, df = system(*case)
    C = random_orbitals(df.nbf, 10, seed=2) * 0.3
    full = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    full.upload_qtri(df.B_tri)
    J0, K0, _ = full.compute(C)
    blocked = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    edges = [0, 7, 40, df.naux]
    for a, b in zip(edges[:-1], edges[1:]):
        blocked.upload_block(df.B_tri[a:b], a)
    J1, K1, _ = blocked.compute(C)
    assert np.array_equal(J0, J1) and np.array_equal(K0, K1)


def test_device_block_upload_and_order(ints_built, jk_built):
    torch = pytest.importorskip("torch")
    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz")
    C = random_orbitals(df.nbf, 10, seed=3) * 0.3
    full = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    full.upload_qtri(df.B_tri)
    J0, K0, _ = full.compute(C)
    eng = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    Bt = torch.from_numpy(np.ascontiguousarray(df.B_tri)).cuda()
    with pytest.raises(GdfjkError):
        eng.upload_device_block(Bt[5:].data_ptr(), 5, df.naux - 5)  # must start at q0 = 0
    half = df.naux // 2
    eng.upload_device_block(Bt.data_ptr(), 0, half)
    with pytest.raises(GdfjkError):
        eng.compute(C)  # not all aux rows uploaded yet
    eng.upload_device_block(Bt[half:].data_ptr(), half, df.naux - half)
    J1, K1, _ = eng.compute(C)
    assert np.array_equal(J0, J1) and np.array_equal(K0, K1)
