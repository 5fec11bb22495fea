"""The bounds-checked engine (libgdfjk_bchk.so, -DGDFJK_BOUNDS_CHECK): every tensor-core path
runs with each bulk-copy source range and global write checked against its buffer's extent.

The checked library is loaded in a child process (the engine library is loaded once per
process); the child runs the paths below, which must finish without a GDFJK_BOUNDS report or a
device error flag, and writes its results; the parent runs the same paths through the release
library and compares.  The checks only skip out-of-range accesses, so on correct index
arithmetic the two libraries compute the same numbers.

Paths: the emulated half-transform, split of X, contraction and reduction (one aux batch and
several, through a small X budget), the non-symmetric emulated K (second digit copy of C and
X), the split-precision full and incremental builds (transform, contraction, reduction), and
the general tensor-core product in both operand orders with a column chunk budget that splits
the product."""
import os
import subprocess
import sys

import numpy as np
import pytest

from psi4_gb300 import _jkabi as abi

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
EMU = abi.DO_J | abi.DO_K | abi.EMULATED


def run_paths() -> dict:
    """Every checked path once, on (H2O)_8 cc-pVDZ real integrals and seeded random operands."""
    import torch

    from psi4_gb300.jk import DFJKEngine, density_difference_factor
    from tests.helpers import random_orbitals, system

    mol, pb, ab, ints, df = system("h2o_8", "cc-pvdz")
    eng = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask)
    eng.upload_pqq(df.to_pQq(), df.sparsity)
    nocc = 20
    C = random_orbitals(df.nbf, nocc, seed=3) * 0.3
    C2 = C + 0.01 * random_orbitals(df.nbf, nocc, seed=5)
    Cr = random_orbitals(df.nbf, nocc, seed=4) * 0.3
    out = {}
    out["emu_J"], out["emu_K"], _ = eng.compute(C, mode=EMU)
    old = os.environ.get("GDFJK_OZ_XCAP_GB")
    os.environ["GDFJK_OZ_XCAP_GB"] = "0.002"  # several aux batches
    try:
        out["emu_K_batched"] = eng.compute(C, mode=EMU)[1]
        out["emu_K_nonsym"] = eng.compute(C, Cr, mode=EMU)[1]
    finally:
        if old is None:
            os.environ.pop("GDFJK_OZ_XCAP_GB")
        else:
            os.environ["GDFJK_OZ_XCAP_GB"] = old
    out["mixed_K0"] = eng.compute_incremental(C, C, nocc, mode=abi.DO_K | abi.MIXED, reset=True)[1]
    U, npos = density_difference_factor(C2, C)
    out["mixed_K1"] = eng.compute_incremental(C2, U, npos, mode=abi.DO_K | abi.MIXED)[1]
    dev = torch.device("cuda:0")
    g = torch.Generator(device=dev)
    g.manual_seed(11)
    M, N, K = 300, 277, 1500
    A = torch.randn((M, K), dtype=torch.float64, device=dev, generator=g)
    Bn = torch.randn((K, N), dtype=torch.float64, device=dev, generator=g)
    Bt = torch.randn((N, K), dtype=torch.float64, device=dev, generator=g)
    for name, Bm, transb in (("gemm_nn", Bn, False), ("gemm_nt", Bt, True)):
        Cm = torch.empty((M, N), dtype=torch.float64, device=dev)
        eng.gemm(A.data_ptr(), K, Bm.data_ptr(), K if transb else N, Cm.data_ptr(), N, M, N, K, transb=transb)
        out[name] = Cm.cpu().numpy()
    old = os.environ.get("GDFJK_OZ_GEMM_CHUNK_GB")
    os.environ["GDFJK_OZ_GEMM_CHUNK_GB"] = "0.0001"  # column chunks of 128
    try:
        Cm = torch.empty((M, N), dtype=torch.float64, device=dev)
        eng.gemm(A.data_ptr(), K, Bn.data_ptr(), N, Cm.data_ptr(), N, M, N, K)
        out["gemm_chunked"] = Cm.cpu().numpy()
    finally:
        if old is None:
            os.environ.pop("GDFJK_OZ_GEMM_CHUNK_GB")
        else:
            os.environ["GDFJK_OZ_GEMM_CHUNK_GB"] = old
    eng.close()
    return out


def test_bounds_checked_library_matches_release(jk_built, tmp_path):
    from psi4_gb300 import _native

    _native.build_jk(bounds_check=True)
    path = tmp_path / "checked.npz"
    env = dict(os.environ, GDFJK_BOUNDS_CHECK="1")
    code = ("import sys, numpy as np; sys.path.insert(0, %r); from tests.test_gpu_bounds_check import run_paths; "
            "from psi4_gb300 import _native; out = run_paths(); print('library', _native.jk_lib()._name); "
            "np.savez(%r, **out)") % (ROOT, str(path))
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, env=env, stdout=subprocess.PIPE,
                       stderr=subprocess.STDOUT, text=True, timeout=900)
    print(r.stdout[-4000:])
    assert r.returncode == 0, "checked run failed"
    assert "GDFJK_BOUNDS" not in r.stdout
    assert "libgdfjk_bchk.so" in r.stdout  # the child ran the checked library
    checked = dict(np.load(path))
    release = run_paths()
    assert set(checked) == set(release)
    for k in sorted(release):
        d = np.abs(checked[k] - release[k]).max()
        print(f"{k}: max|checked - release| {d:.2e} (scale {np.abs(release[k]).max():.2e})")
        assert d <= 1e-12 * max(1.0, np.abs(release[k]).max()), k
