"""The J passes on the engine's second stream.

With a tensor-core K and at least 8 GB of B the two J passes run on their own stream beside K
and join K's stream at the end of the build; below that, and beside the native FP64 K, they run
on K's stream.  The same kernels form the same sums on either stream, so on one B every path
gives bitwise the same J and K:

* a J+K emulated build (J beside K) against a J-only and a K-only build;
* the precision form's emulated FP64 anchor (a J-only build left unjoined, then a K-only build
  on the C that the J build padded) against the plain build;
* D handed back by the J+K build against C C^T."""
import numpy as np
import pytest

from psi4_gb300 import _jkabi as abi

pytestmark = pytest.mark.gpu


def test_forked_j_paths_agree(jk_built):
    import torch

    from psi4_gb300.jk import DFJKEngine
    from tests.helpers import random_orbitals

    nbf, naux, nocc = 1024, 1920, 48
    npair = nbf * (nbf + 1) // 2
    # 1920 aux rows x 136 stored tiles x 32 KB = 8.56 GB of B: above the second-stream threshold
    assert naux * (nbf // 64) * (nbf // 64 + 1) // 2 * 4096 * 8 >= 8e9
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev)
    g.manual_seed(21)
    eng = DFJKEngine(nbf, naux, None)
    B = torch.empty((naux, npair), dtype=torch.float64, device=dev)
    for q0 in range(0, naux, 256):
        B[q0:q0 + 256].normal_(0.0, 0.02, generator=g)
    torch.cuda.synchronize()
    eng.upload_device(B.data_ptr())
    del B
    torch.cuda.empty_cache()
    C = random_orbitals(nbf, nocc, seed=7) * 0.1
    try:
        J1, K1, D1 = eng.compute(C, mode=abi.DO_J | abi.DO_K | abi.EMULATED, want_D=True)
        J2 = eng.compute(C, mode=abi.DO_J)[0]
        K2 = eng.compute(C, mode=abi.DO_K | abi.EMULATED)[1]
        J3, K3 = eng.compute_incremental(C, C, nocc, mode=abi.DO_J | abi.DO_K | abi.EMULATED)
    finally:
        eng.close()
    assert np.array_equal(J1, J2) and np.array_equal(J1, J3)
    assert np.array_equal(K1, K2) and np.array_equal(K1, K3)
    assert np.abs(D1 - C @ C.T).max() < 1e-13
    assert np.abs(J1).max() > 0 and np.abs(K1).max() > 0
