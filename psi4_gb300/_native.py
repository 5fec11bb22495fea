"""In-tree build and loading of the native libraries.

* ``libgdfints.so`` — host integral provider (C++/OpenMP, g++), include/gdfints.h.
* ``libgdfjk.so``   — the GB300 DF-JK engine (CUDA for sm_103a + C++ host), include/gdfjk.h.

Both are compiled into ``psi4_gb300/lib/`` (git-ignored).  Loading never falls back to
anything else: a missing library raises.
"""
from __future__ import annotations

import ctypes
import os
import shutil
import subprocess
import threading
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
LIB = os.path.join(PKG, "lib")
INC = os.path.join(ROOT, "include")
CSRC = os.path.join(PKG, "csrc")

INTS_SO = os.path.join(LIB, "libgdfints.so")
JK_SO = os.path.join(LIB, "libgdfjk.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
JK_SOURCES = ["gdfjk_host.cu", "j_kernels.cu", "k_fp64.cu", "k_mixed.cu", "k_oz.cu", "backward.cu", "noalloc.cu"]

_lock = threading.Lock()


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libgdfjk.so")
    return cand


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout)
    return r.stdout


def build_ints(force: bool = False) -> str:
    os.makedirs(LIB, exist_ok=True)
    src = os.path.join(CSRC, "ints", "gdf_ints.cpp")
    if force or not os.path.exists(INTS_SO) or os.path.getmtime(INTS_SO) < os.path.getmtime(src):
        _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-I", INC, "-o", INTS_SO + ".tmp", src])
        os.replace(INTS_SO + ".tmp", INTS_SO)
    return INTS_SO


def _jk_sources():
    return [os.path.join(CSRC, "jk", s) for s in JK_SOURCES if os.path.exists(os.path.join(CSRC, "jk", s))]


def build_jk(force: bool = False, extra_flags=None) -> str:
    os.makedirs(LIB, exist_ok=True)
    srcs = _jk_sources()
    hdrs = [os.path.join(CSRC, "jk", h) for h in os.listdir(os.path.join(CSRC, "jk")) if h.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(INC, "gdfjk.h"))
    newest = max(os.path.getmtime(p) for p in srcs + hdrs)
    if not force and os.path.exists(JK_SO) and os.path.getmtime(JK_SO) >= newest:
        return JK_SO
    nvcc = _nvcc()
    objdir = os.path.join(LIB, "obj")
    os.makedirs(objdir, exist_ok=True)
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INC, "--expt-relaxed-constexpr"]
    flags += list(extra_flags or [])

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        _run([nvcc] + flags + ["-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    _run([nvcc] + ARCH + ["-shared", "-o", JK_SO + ".tmp"] + objs)
    os.replace(JK_SO + ".tmp", JK_SO)
    return JK_SO


_ints = None
_jk = None


def ints_lib() -> ctypes.CDLL:
    global _ints
    with _lock:
        if _ints is None:
            if not os.path.exists(INTS_SO):
                build_ints()
            _ints = ctypes.CDLL(INTS_SO)
            _declare_ints(_ints)
        return _ints


def jk_lib() -> ctypes.CDLL:
    """Load libgdfjk.so.  Raises if it has not been built: there is no other JK path."""
    global _jk
    with _lock:
        if _jk is None:
            if not os.path.exists(JK_SO):
                raise RuntimeError(
                    f"{JK_SO} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`"
                )
            _jk = ctypes.CDLL(JK_SO)
            _declare_jk(_jk)
        return _jk


P = ctypes.c_void_p
I = ctypes.c_int
D = ctypes.c_double
SZ = ctypes.c_size_t


def _declare_ints(L):
    L.gdfints_last_error.restype = ctypes.c_char_p
    L.gdfints_basis_create.argtypes = [I, P, P, P, P, P, P, P, I, ctypes.POINTER(P)]
    L.gdfints_basis_destroy.argtypes = [P]
    L.gdfints_basis_destroy.restype = None
    L.gdfints_basis_nbf.argtypes = [P]
    for name, args in [
        ("gdfints_overlap", [P, P]),
        ("gdfints_kinetic", [P, P]),
        ("gdfints_potential", [P, I, P, P, P]),
        ("gdfints_metric", [P, P]),
        ("gdfints_schwarz", [P, P, P]),
        ("gdfints_three_index", [P, P, P, I, I, P]),
        ("gdfints_three_index_erf", [P, P, P, I, I, D, P]),
        ("gdfints_overlap_grad", [P, P, I, P]),
        ("gdfints_kinetic_grad", [P, P, I, P]),
        ("gdfints_potential_grad", [P, P, I, P, P, P]),
        ("gdfints_metric_grad", [P, P, I, P]),
        ("gdfints_three_index_grad", [P, P, P, P, I, P]),
        ("gdfints_boys", [I, D, P]),
    ]:
        f = getattr(L, name)
        f.argtypes = args
        f.restype = I


def _declare_jk(L):
    from . import _jkabi

    _jkabi.declare(L)
