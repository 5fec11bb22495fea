"""The allocation-free Coulomb entry point (gdfjk_coulomb_noalloc) against the regular one.

It exists for callers that cannot call cudaMalloc (code running inside another framework's
memory pool or allocator hooks, hosts that forbid allocation after start-up, drivers that
fix their buffers once): they hand in B, D and J, and the fitted density d_Q lives in a
fixed device array inside the library.  This file is collected last on purpose; it needs
nothing from the other tests and passes alone in a fresh process too.
"""
import ctypes

import numpy as np
import pytest

from psi4_gb300 import _jkabi as abi
from psi4_gb300 import _native
from psi4_gb300.jk import DFJKEngine
from tests.helpers import random_orbitals, system

pytestmark = pytest.mark.gpu
TOL = 1e-10  # plus 1e-14 of max|J|: random orbitals drive J far above physical magnitudes


def _noalloc(L, nbf, naux, B, D, J, stream):
    return L.gdfjk_coulomb_noalloc(nbf, naux, ctypes.c_void_p(B.data_ptr()), ctypes.c_void_p(D.data_ptr()),
                                   ctypes.c_void_p(J.data_ptr()), ctypes.c_void_p(stream))


@pytest.mark.parametrize("case", [("h2o_2", "cc-pvdz", 1e-12), ("h2o_8", "cc-pvdz", 1e-12)])
def test_noalloc_matches_regular_entry_point(ints_built, jk_built, case):
    torch = pytest.importorskip("torch")
    mol, pb, ab, ints, df = system(*case)
    nbf, naux = df.nbf, df.naux
    L = _native.jk_lib()
    eng = DFJKEngine(nbf, naux, None)
    eng.upload_qtri(df.B_tri)
    Bd = torch.from_numpy(np.ascontiguousarray(df.B_tri)).cuda()
    J = torch.empty((nbf, nbf), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    for call, seed in enumerate((21, 22)):  # two calls in a row, different densities
        C = random_orbitals(nbf, 9 + call, seed)
        Dd = torch.from_numpy(C @ C.T).cuda()
        rc = _noalloc(L, nbf, naux, Bd, Dd, J, stream)
        assert rc == 0, L.gdfjk_last_error(None).decode()
        torch.cuda.synchronize()
        Jref, _, _ = eng.compute(C, mode=abi.DO_J)
        assert np.abs(J.cpu().numpy() - Jref).max() < TOL + 1e-14 * np.abs(Jref).max()


def test_noalloc_allocates_nothing_and_symmetrises_D(ints_built, jk_built):
    """A warmed call leaves the device's free memory unchanged, and a non-symmetric D gives
    the J of its symmetric part (D + D^T)/2, as the header states."""
    torch = pytest.importorskip("torch")
    mol, pb, ab, ints, df = system("h2o_2", "cc-pvdz", 1e-12)
    nbf, naux = df.nbf, df.naux
    L = _native.jk_lib()
    eng = DFJKEngine(nbf, naux, None)
    eng.upload_qtri(df.B_tri)
    Bd = torch.from_numpy(np.ascontiguousarray(df.B_tri)).cuda()
    rng = np.random.default_rng(5)
    Dn = rng.standard_normal((nbf, nbf)) * 0.05  # not symmetric
    Dd = torch.from_numpy(Dn).cuda()
    J = torch.empty((nbf, nbf), dtype=torch.float64, device="cuda")
    stream = torch.cuda.current_stream().cuda_stream
    assert _noalloc(L, nbf, naux, Bd, Dd, J, stream) == 0  # warm: the module is loaded
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    assert _noalloc(L, nbf, naux, Bd, Dd, J, stream) == 0, L.gdfjk_last_error(None).decode()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    # reference: the regular entry point on the symmetric part, through a signed factor of it
    Ds = 0.5 * (Dn + Dn.T)
    w, V = np.linalg.eigh(Ds)
    Cp = V[:, w > 0] * np.sqrt(w[w > 0])
    Cm = V[:, w < 0] * np.sqrt(-w[w < 0])
    Jp, _, _ = eng.compute(Cp, mode=abi.DO_J)
    Jm, _, _ = eng.compute(Cm, mode=abi.DO_J)
    Jref = Jp - Jm
    assert np.abs(J.cpu().numpy() - Jref).max() < TOL + 1e-14 * np.abs(Jref).max()


def test_noalloc_rejects_oversized_naux(jk_built):
    L = _native.jk_lib()
    big = abi.NOALLOC_MAX_NAUX + 1
    dummy = ctypes.c_void_p(16)  # never dereferenced: the size check comes first
    rc = L.gdfjk_coulomb_noalloc(10, big, dummy, dummy, dummy, None)
    assert rc == abi.GDFJK_ERR_ARG
    assert b"exceeds" in L.gdfjk_last_error(None)
