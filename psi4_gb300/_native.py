"""In-tree build and loading of the native libraries.

* ``libgdfints.so`` — host integral provider (C++/OpenMP, g++), include/gdfints.h.
* ``libgdfjk.so``   — the GB300 DF-JK engine (CUDA for sm_103a + C++ host), include/gdfjk.h.
* ``libgdfjk_bchk.so`` — the same engine compiled with -DGDFJK_BOUNDS_CHECK: every bulk-copy
  source range and global write of the tensor-core kernels is checked against its buffer's
  extent (a violation sets the device error flag, GDFJK_ERR_DEVICE, instead of faulting).
  Built on request (``build_jk(bounds_check=True)``) and loaded instead of libgdfjk.so when
  GDFJK_BOUNDS_CHECK=1 is set in the environment before the first load.

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
JK_BCHK_SO = os.path.join(LIB, "libgdfjk_bchk.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# ints3c_lc*.cu (the integral class kernels) come first: they take the longest to compile
JK_SOURCES = ["ints3c_lc2.cu", "ints3c_lc3.cu", "ints3c_lc1.cu", "ints3c_lc4.cu", "ints3c_lc0.cu", "k_oz.cu", "k_mixed.cu",
              "gdfjk_host.cu", "j_kernels.cu", "k_fp64.cu", "backward.cu", "noalloc.cu", "ints3c.cu"]

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
    newest = max(os.path.getmtime(p) for p in (src, os.path.join(CSRC, "ints", "gto_tables.h")))
    if force or not os.path.exists(INTS_SO) or os.path.getmtime(INTS_SO) < newest:
        _run(["g++", "-O3", "-std=c++17", "-fopenmp", "-fPIC", "-shared", "-I", INC, "-o", INTS_SO + ".tmp", src])
        os.replace(INTS_SO + ".tmp", INTS_SO)
    return INTS_SO


def _jk_sources():
    return [os.path.join(CSRC, "jk", s) for s in JK_SOURCES if os.path.exists(os.path.join(CSRC, "jk", s))]


def build_jk(force: bool = False, extra_flags=None, bounds_check: bool = False) -> str:
    """Compile libgdfjk.so (or, with `bounds_check`, libgdfjk_bchk.so) unless it is newer than
    every source and header."""
    os.makedirs(LIB, exist_ok=True)
    out = JK_BCHK_SO if bounds_check else JK_SO
    srcs = _jk_sources()
    hdrs = [os.path.join(CSRC, "jk", h) for h in os.listdir(os.path.join(CSRC, "jk")) if h.endswith((".cuh", ".h"))]
    hdrs.append(os.path.join(INC, "gdfjk.h"))
    hdrs.append(os.path.join(CSRC, "ints", "gto_tables.h"))
    newest = max(os.path.getmtime(p) for p in srcs + hdrs)
    if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    nvcc = _nvcc()
    objdir = os.path.join(LIB, "obj_bchk" if bounds_check else "obj")
    os.makedirs(objdir, exist_ok=True)
    flags = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INC, "--expt-relaxed-constexpr"]
    if bounds_check:
        flags.append("-DGDFJK_BOUNDS_CHECK")
    flags += list(extra_flags or [])

    def compile_one(src):
        obj = os.path.join(objdir, os.path.basename(src) + ".o")
        _run([nvcc] + flags + ["-c", src, "-o", obj])
        return obj

    with ThreadPoolExecutor(max_workers=min(max(4, os.cpu_count() or 4), len(srcs))) as ex:
        objs = list(ex.map(compile_one, srcs))
    _run([nvcc] + ARCH + ["-shared", "-o", out + ".tmp"] + objs)
    os.replace(out + ".tmp", out)
    return out


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
    """Load libgdfjk.so (libgdfjk_bchk.so when GDFJK_BOUNDS_CHECK=1).  Raises if it has not
    been built: there is no other JK path."""
    global _jk
    with _lock:
        if _jk is None:
            checked = os.environ.get("GDFJK_BOUNDS_CHECK", "0") == "1"
            path = JK_BCHK_SO if checked else JK_SO
            if not os.path.exists(path):
                how = "_native.build_jk(bounds_check=True)" if checked else "import __graft_entry__ as g; g.build()"
                raise RuntimeError(f"{path} is missing: build it with `python -c '{how}'`")
            _jk = ctypes.CDLL(path)
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
