"""B kept in pinned Grace memory (GDFJK_B_HOST): the same kernels read it over NVLink-C2C, so
every form gives bitwise the results of the HBM-resident engine — psi4's out-of-core
DFHelper path (grab_AO, dfhelper.cc:1419-1432) without a second code path."""
import numpy as np
import pytest

from psi4_gb300 import _jkabi as abi
from psi4_gb300.jk import DFJKEngine
from tests.helpers import random_orbitals, system

pytestmark = pytest.mark.gpu


def _engines(df, flags_a=0, flags_b=abi.B_HOST):
    out = []
    for fl in (flags_a, flags_b):
        eng = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask, flags=fl)
        eng.upload_pqq(df.to_pQq(), df.sparsity)
        out.append(eng)
    return out


@pytest.mark.parametrize("mode_name", ["fp64", "emulated", "mixed"])
def test_host_b_matches_device_b(ints_built, jk_built, mode_name):
    mol, pb, ab, ints, df = system("h2o_8", "cc-pvdz")
    dev, host = _engines(df)
    C = random_orbitals(df.nbf, 40, seed=2) * 0.3
    mode = abi.DO_J | abi.DO_K | {"fp64": 0, "emulated": abi.EMULATED, "mixed": abi.MIXED}[mode_name]
    Jd, Kd, _ = dev.compute(C, mode=mode)
    Jh, Kh, _ = host.compute(C, mode=mode)
    assert np.array_equal(Jd, Jh)
    assert np.array_equal(Kd, Kh)


def test_host_b_nonsymmetric_and_backward(ints_built, jk_built):
    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz")
    dev, host = _engines(df)
    Cl = random_orbitals(df.nbf, 9, seed=3)
    Cr = random_orbitals(df.nbf, 9, seed=4)
    a = dev.compute(Cl, Cr, mode=abi.DO_J | abi.DO_K)
    b = host.compute(Cl, Cr, mode=abi.DO_J | abi.DO_K)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    rng = np.random.default_rng(5)
    gJ = rng.standard_normal((df.nbf, df.nbf))
    gK = rng.standard_normal((df.nbf, df.nbf))
    dC1, G1 = dev.backward(Cl, gJ, gK)
    dC2, G2 = host.backward(Cl, gJ, gK)
    assert np.array_equal(dC1, dC2) and np.array_equal(G1, G2)


def test_host_b_block_upload_and_memory_query(jk_built):
    """Blocks uploaded from the device land in host memory; the memory query leaves B out."""
    torch = pytest.importorskip("torch")
    nbf, naux, nocc = 200, 48, 24
    dev_ = torch.device("cuda:0")
    g = torch.Generator(device=dev_)
    g.manual_seed(9)
    Bt = torch.randn((naux, nbf * (nbf + 1) // 2), dtype=torch.float64, device=dev_, generator=g) * 0.05
    e1 = DFJKEngine(nbf, naux, None)
    e1.upload_device(Bt.data_ptr())
    e2 = DFJKEngine(nbf, naux, None, flags=abi.B_HOST)
    e2.upload_device_block(Bt.data_ptr(), 0, 20)
    e2.upload_device_block(Bt[20:].data_ptr(), 20, naux - 20)
    C = np.random.default_rng(1).standard_normal((nbf, nocc)) * 0.2
    for mode in (abi.DO_J | abi.DO_K, abi.DO_J | abi.DO_K | abi.EMULATED):
        r1 = e1.compute(C, mode=mode)
        r2 = e2.compute(C, mode=mode)
        assert np.array_equal(r1[0], r2[0]) and np.array_equal(r1[1], r2[1])
    full = DFJKEngine.query_memory(nbf, naux, nocc, 0)
    no_b = DFJKEngine.query_memory(nbf, naux, nocc, abi.B_HOST)
    ntiles = (nbf + 63) // 64 * ((nbf + 63) // 64 + 1) // 2
    assert full - no_b == naux * ntiles * 4096 * 8
