"""Argument checks of the device integral entries that run before any device work (CPU)."""
import ctypes

import numpy as np
import pytest

from psi4_gb300 import _jkabi, _native


def _create(L, l, puream=1):
    n = len(l)
    la = np.array(l, dtype=np.int32)
    npr = np.ones(n, dtype=np.int32)
    off = np.arange(n, dtype=np.int32)
    ex = np.ones(n)
    cf = np.ones(n)
    xyz = np.zeros(3 * n)
    h = ctypes.c_void_p()
    p = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    return L.gdfjk_basis_create(0, n, p(la), p(npr), p(off), p(ex), p(cf), p(xyz), None, puream, ctypes.byref(h)), h


def test_basis_create_rejects_h_shells(jk_built):
    L = _native.jk_lib()
    rc, _ = _create(L, [0, 1, 5])
    assert rc == _jkabi.GDFJK_ERR_ARG
    assert b"above g" in L.gdfjk_last_error(None)


def test_three_index_rejects_null_bases(jk_built):
    L = _native.jk_lib()
    rc = L.gdfjk_three_index_device(None, None, None, 0, 1, None, 1, None, None)
    assert rc == _jkabi.GDFJK_ERR_ARG
    rc = L.gdfjk_metric_device(None, 0, 1, 1, None, None)
    assert rc == _jkabi.GDFJK_ERR_ARG
    assert L.gdfjk_three_index_grad_device(None, None, None, None, None, 1, 1, None, None) == _jkabi.GDFJK_ERR_ARG
    assert L.gdfjk_metric_grad_device(None, None, 1, 1, None, None) == _jkabi.GDFJK_ERR_ARG
