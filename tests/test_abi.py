"""The C-ABI libraries load on the CPU and export every function their headers declare."""
import ctypes
import os
import re

from psi4_gb300 import _jkabi, _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared(header, prefix):
    text = open(os.path.join(ROOT, "include", header)).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(" + prefix + r"_\w+)\s*\(", text)))


def test_gdfjk_exports_every_declared_symbol(jk_built):
    lib = ctypes.CDLL(_native.JK_SO)
    names = _declared("gdfjk.h", "gdfjk")
    assert names, "no declarations parsed"
    for n in names:
        assert hasattr(lib, n), n
    # the ctypes signature table covers the whole header
    assert sorted(_jkabi.SIGNATURES) == names


def test_bounds_checked_build_exports_every_declared_symbol(jk_built):
    """-DGDFJK_BOUNDS_CHECK compiles (the checks are live in this build) into its own library
    with the same interface."""
    path = _native.build_jk(bounds_check=True)
    assert path == _native.JK_BCHK_SO and path != _native.JK_SO
    lib = ctypes.CDLL(path)
    for n in _declared("gdfjk.h", "gdfjk"):
        assert hasattr(lib, n), n


def test_gdfints_exports_every_declared_symbol(ints_built):
    lib = ctypes.CDLL(_native.INTS_SO)
    for n in _declared("gdfints.h", "gdfints"):
        assert hasattr(lib, n), n


def test_query_memory_without_gpu(jk_built):
    from psi4_gb300.jk import DFJKEngine

    b = DFJKEngine.query_memory(1856, 4448, 160)
    # B tiles alone are naux * 435 tiles * 32 KB
    assert b > 4448 * 435 * 4096 * 8


def test_create_rejects_bad_sizes_without_gpu(jk_built):
    L = _native.jk_lib()
    h = ctypes.c_void_p()
    assert L.gdfjk_create(0, 0, 10, None, 0, ctypes.byref(h)) == _jkabi.GDFJK_ERR_ARG
    assert b"positive" in L.gdfjk_last_error(None)


def test_query_memory_leaves_host_b_out_without_gpu(jk_built):
    """With GDFJK_B_HOST the FP64 tiles of B live in host memory: the device estimate drops
    by exactly their bytes (C2 shape, dense: 435 stored tiles)."""
    from psi4_gb300.jk import DFJKEngine

    full = DFJKEngine.query_memory(1856, 4448, 160)
    host = DFJKEngine.query_memory(1856, 4448, 160, _jkabi.B_HOST)
    assert full - host == 4448 * 435 * 4096 * 8


def test_memory_estimate_counts_wk_tensors_without_gpu(jk_built):
    """GpuDFJK.memory_estimate (doubles, like JK::memory_estimate) adds the two wK tensors."""
    from types import SimpleNamespace

    from psi4_gb300.jk import GpuDFJK

    jk = GpuDFJK(df_tensor=SimpleNamespace(nbf=384, naux=1856))
    base = jk.memory_estimate()
    jk.set_do_wK(True)
    b_tiles = 1856 * (6 * 7 // 2) * 4096  # doubles of one tensor in tiles
    assert jk.memory_estimate() - base == 2 * b_tiles
