"""B = J^-1/2 (P|mn) built on the device for large systems (the caller's initialisation).

This is psi4's ``DFHelper::prepare_AO_core`` (psi4/src/psi4/lib3index/dfhelper.cc:514-588)
arranged for one GB300: the raw 3-index integrals (P|mn) of the Schwarz-significant shell
pairs (``compute_sparse_pQq_blocking_p_symm``, dfhelper.cc:1284-1347) and the metric (P|Q)
(``FittingMetric::form_fitting_metric``, fittingmetric.cc:72) are computed by the engine's
integral kernels straight into device arrays (``gdfjk_three_index_device``,
``gdfjk_metric_device``; ``device_integrals=False`` takes them from the host provider
instead, in blocks of aux rows); the metric contraction (``contract_metric_AO_core_symm``,
dfhelper.cc:1653-1678) runs on the tensor cores to FP64 accuracy
(``gdfjk_metric_contract_device``); B is then relaid into the engine's tiles
(``gdfjk_upload_B_device``).  Screening (the Schwarz diagonal) and the metric power are the
host restatements of ``dfhelper.py`` (prepare_sparsity, Matrix::power).

torch supplies the device arrays (plumbing); every computation on them is the engine's.
"""
from __future__ import annotations

import ctypes
import time
from dataclasses import dataclass, field

import numpy as np

from .basis import BasisSet
from .dfhelper import DEFAULT_CONDITION, DEFAULT_CUTOFF, Sparsity, metric_power, prepare_sparsity
from .ints import Integrals
from .jk import DFJKEngine, GdfjkError
from .molecule import Molecule


class DeviceBasis:
    """A basis set copied to a CUDA device for the engine's integral kernels
    (gdfjk_basis_create): shells, primitives and normalised contraction coefficients."""

    def __init__(self, bs: BasisSet, device: int = 0):
        from . import _native

        self.L = _native.jk_lib()
        self.bs = bs
        self.device = device
        self._keep = [np.ascontiguousarray(x) for x in (bs.l.astype(np.int32), bs.nprim.astype(np.int32),
                                                        bs.prim_offset.astype(np.int32), bs.exps, bs.coefs,
                                                        bs.centers.reshape(-1), bs.atom.astype(np.int32))]
        l, npr, off, ex, cf, xyz, at = self._keep
        h = ctypes.c_void_p()
        rc = self.L.gdfjk_basis_create(int(device), bs.nshell, _p(l), _p(npr), _p(off), _p(ex), _p(cf), _p(xyz), _p(at),
                                       int(bs.puream), ctypes.byref(h))
        if rc != 0:
            raise GdfjkError(rc, self.L.gdfjk_last_error(None).decode())
        self.h = h
        self.nbf = self.L.gdfjk_basis_nbf(h)
        assert self.nbf == bs.nbf

    def close(self):
        if getattr(self, "h", None):
            self.L.gdfjk_basis_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def three_index_device(aux: DeviceBasis, prim: DeviceBasis, out_ptr: int, ldo: int, shell_mask=None, p0: int = 0,
                       p1: int | None = None, col_map_ptr: int | None = None, stream: int | None = None):
    """(P|mn), p0 <= P < p1, for the shell pairs M >= N of shell_mask (None: all) into the
    device array at out_ptr (row P - p0 at out_ptr + 8 (P - p0) ldo; column m(m+1)/2+n, or
    col_map[m(m+1)/2+n] when col_map_ptr is given).  Unlisted pairs are not written."""
    p1 = aux.nbf if p1 is None else p1
    mask = None if shell_mask is None else np.ascontiguousarray(shell_mask, dtype=np.uint8)
    rc = aux.L.gdfjk_three_index_device(aux.h, prim.h, None if mask is None else _p(mask), int(p0), int(p1),
                                        None if col_map_ptr is None else ctypes.c_void_p(col_map_ptr), int(ldo),
                                        ctypes.c_void_p(out_ptr), None if not stream else ctypes.c_void_p(stream))
    if rc != 0:
        raise GdfjkError(rc, aux.L.gdfjk_last_error(None).decode())


def three_index_grad_device(aux: DeviceBasis, prim: DeviceBasis, G3_ptr: int, ldg: int, natom: int, grad_ptr: int,
                            shell_mask=None, col_map_ptr: int | None = None, stream: int | None = None):
    """grad[natom][3] (device, accumulated) += sum G3[P][col(m,n)] d(P|mn)/dx over the shell
    pairs of shell_mask (gdfjk_three_index_grad_device)."""
    mask = None if shell_mask is None else np.ascontiguousarray(shell_mask, dtype=np.uint8)
    rc = aux.L.gdfjk_three_index_grad_device(aux.h, prim.h, None if mask is None else _p(mask), ctypes.c_void_p(G3_ptr),
                                             None if col_map_ptr is None else ctypes.c_void_p(col_map_ptr), int(ldg),
                                             int(natom), ctypes.c_void_p(grad_ptr),
                                             None if not stream else ctypes.c_void_p(stream))
    if rc != 0:
        raise GdfjkError(rc, aux.L.gdfjk_last_error(None).decode())


def potential_grad_device(prim: DeviceBasis, Dp_ptr: int, mol: Molecule, grad_ptr: int, stream: int | None = None):
    """grad[natom][3] (device, accumulated) += sum_{m>=n} Dp[m(m+1)/2+n] dV_mn/dx, the nuclear
    attraction's derivative integrals with the molecule's point charges
    (gdfjk_potential_grad_device); Dp: device packed triangle, off-diagonal entries doubled."""
    Z = np.ascontiguousarray(mol.Z, dtype=np.float64)
    xyz = np.ascontiguousarray(mol.xyz, dtype=np.float64).reshape(-1)
    rc = prim.L.gdfjk_potential_grad_device(prim.h, ctypes.c_void_p(Dp_ptr), int(mol.natom), _p(Z), _p(xyz),
                                            ctypes.c_void_p(grad_ptr), None if not stream else ctypes.c_void_p(stream))
    if rc != 0:
        raise GdfjkError(rc, prim.L.gdfjk_last_error(None).decode())


def metric_grad_device(aux: DeviceBasis, G2_ptr: int, ldg: int, natom: int, grad_ptr: int, stream: int | None = None):
    """grad[natom][3] (device, accumulated) += sum G2[P][Q] d(P|Q)/dx (gdfjk_metric_grad_device)."""
    rc = aux.L.gdfjk_metric_grad_device(aux.h, ctypes.c_void_p(G2_ptr), int(ldg), int(natom), ctypes.c_void_p(grad_ptr),
                                        None if not stream else ctypes.c_void_p(stream))
    if rc != 0:
        raise GdfjkError(rc, aux.L.gdfjk_last_error(None).decode())


def metric_device(aux: DeviceBasis, out_ptr: int, ldo: int, p0: int = 0, p1: int | None = None,
                  stream: int | None = None):
    """The Coulomb metric (P|Q), rows p0 <= P < p1, into the device array at out_ptr."""
    p1 = aux.nbf if p1 is None else p1
    rc = aux.L.gdfjk_metric_device(aux.h, int(p0), int(p1), int(ldo), ctypes.c_void_p(out_ptr),
                                   None if not stream else ctypes.c_void_p(stream))
    if rc != 0:
        raise GdfjkError(rc, aux.L.gdfjk_last_error(None).decode())


@dataclass
class DeviceDF:
    engine: DFJKEngine
    nbf: int
    naux: int
    sparsity: Sparsity
    metric: np.ndarray       # (P|Q)
    Jmhalf: np.ndarray       # J^-1/2 with psi4's eigenvalue truncation
    ints: Integrals
    timings: dict = field(default_factory=dict)
    rows: np.ndarray | None = None  # the first `keep_rows` rows of B (packed triangle), host copy
    metric_eig: tuple | None = None  # (eigenvalues, eigenvectors) of the metric on the device, when computed there


def metric_power_device(Md, power: float, condition: float, eig=None):
    """Matrix::power (matrix.cc:2370-2415) of a device matrix, with the host restatement's
    rule (dfhelper.metric_power): eigendecompose (the library's FP64 symmetric eigensolver),
    drop |lambda| < condition * max|lambda| for negative powers, rebuild V diag(lambda^p) V^T.
    eig: a list that receives (w, V)."""
    import torch

    w, V = torch.linalg.eigh(Md)
    if eig is not None:
        eig[:] = [w, V]
    max_a = torch.maximum(w[-1].abs(), w[0].abs())
    a = torch.where(w > 0, w.clamp(min=torch.finfo(w.dtype).tiny) ** power, torch.zeros_like(w))
    if power < 0.0:
        a = torch.where(w.abs() < condition * max_a, torch.zeros_like(a), a)
    a = torch.where(torch.isfinite(a), a, torch.zeros_like(a))
    return (V * a) @ V.T


# "auto": the device eigensolver from this many fitting functions on (measured on GB300 against
# the 16 host cores: n = 4448 host 1.45 s / device 0.74 s plus ~3.5 s of the library's set-up
# on first use; n = 7424 6.9 / 2.9 s; n = 11646 27.6 / 10.3 s)
METRIC_POWER_DEVICE_FROM = 6000


def _metric_and_power(ints, aux_dev, naux, condition, dev, timings, power_on="auto"):
    """(P|Q) (on the device when aux_dev is given) and J^-1/2 (Matrix::power on the host, or
    on the device with power_on="device"; "auto" picks by size); returns (M, J^-1/2 on the
    host, J^-1/2 on the device)."""
    import torch

    if power_on == "auto":
        power_on = "device" if naux >= METRIC_POWER_DEVICE_FROM else "host"

    tm = time.perf_counter()
    if aux_dev is not None:
        Md = torch.empty((naux, naux), dtype=torch.float64, device=dev)
        metric_device(aux_dev, Md.data_ptr(), naux)
    else:
        Md = torch.from_numpy(ints.metric()).to(dev)
    M = Md.cpu().numpy()
    tp = time.perf_counter()
    eig = []
    if power_on == "device":
        Jm = metric_power_device(Md, -0.5, condition, eig=eig)
        Jm_host = Jm.cpu().numpy()
        timings.update({"metric_s": tp - tm, "metric_power_device_s": time.perf_counter() - tp})
    else:
        Jm_host = metric_power(M, -0.5, condition)
        Jm = torch.from_numpy(Jm_host).to(dev).contiguous()
        timings.update({"metric_s": tp - tm, "metric_power_host_s": time.perf_counter() - tp})
    del Md
    timings["metric_eig"] = tuple(eig) if eig else None
    return M, Jm_host, Jm


def build_device_B(mol: Molecule, primary: BasisSet, aux: BasisSet, device: int = 0, cutoff: float = DEFAULT_CUTOFF,
                   condition: float = DEFAULT_CONDITION, ints: Integrals | None = None, block: int = 128,
                   keep_rows: int = 0, check_columns: int = 0, device_integrals: bool = True,
                   metric_power_on: str = "auto") -> DeviceDF:
    """Build B on the device and upload it into a new engine.  `keep_rows` > 0 also returns a
    host copy of B's first rows (for checks against a CPU restatement); `check_columns` > 0
    compares that many columns of the tensor-core metric contraction with the FP64 library
    GEMM and records the largest difference in ``timings``.  device_integrals: (P|mn) and
    (P|Q) from the engine's integral kernels (else from the host provider); metric_power_on:
    "host" (psi4's Matrix::power restated), "device" (the same rule on the library's FP64
    eigensolver) or "auto" (the device from METRIC_POWER_DEVICE_FROM fitting functions)."""
    import torch

    dev = torch.device("cuda", device)
    t0 = time.perf_counter()
    ints = ints or Integrals(mol, primary, aux)
    nbf, naux = primary.nbf, aux.nbf
    timings = {}
    ts = time.perf_counter()
    fun_max, shell_max = ints.schwarz()
    sp = prepare_sparsity(fun_max, shell_max, cutoff, naux)
    timings["schwarz_and_sparsity_host_s"] = time.perf_counter() - ts
    pb_dev = ab_dev = None
    if device_integrals:
        pb_dev, ab_dev = DeviceBasis(primary, device), DeviceBasis(aux, device)
    M, Jm_host, Jm = _metric_and_power(ints, ab_dev, naux, condition, dev, timings, metric_power_on)
    r, c = np.tril_indices(nbf)
    keep = torch.from_numpy(sp.pair_mask[r, c].astype(np.float64)).to(dev)
    npair = keep.numel()
    t_ints = t_copy = 0.0
    if device_integrals:
        ta = time.perf_counter()
        P = torch.zeros((naux, npair), dtype=torch.float64, device=dev)
        three_index_device(ab_dev, pb_dev, P.data_ptr(), npair, shell_mask=sp.shell_mask)
        P *= keep  # screened pairs are absent from psi4's tensor
        torch.cuda.synchronize(dev)
        timings["three_index_device_s"] = time.perf_counter() - ta
        pb_dev.close()
        ab_dev.close()
    else:
        P = torch.empty((naux, npair), dtype=torch.float64, device=dev)
        for p0 in range(0, naux, block):
            p1 = min(naux, p0 + block)
            ta = time.perf_counter()
            A = ints.three_index(shell_mask=sp.shell_mask, p0=p0, p1=p1)
            t_ints += time.perf_counter() - ta
            tb = time.perf_counter()
            P[p0:p1] = torch.from_numpy(A).to(dev) * keep  # screened pairs are absent from psi4's tensor
            torch.cuda.synchronize(dev)
            t_copy += time.perf_counter() - tb
        timings.update({"three_index_host_s": t_ints, "three_index_copy_s": t_copy})
    del keep
    eng = DFJKEngine(nbf, naux, sp.pair_mask, device=device)
    B = torch.empty((naux, npair), dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    tg = time.perf_counter()
    eng.metric_contract(Jm.data_ptr(), P.data_ptr(), npair, B.data_ptr())
    t_gemm = time.perf_counter() - tg
    timings["metric_contraction_device_s"] = t_gemm
    if check_columns > 0:
        nc = min(npair, check_columns)
        (Jm @ P[:, :1024]).sum().item()  # the library GEMM's first-call set-up stays out of its time
        torch.cuda.synchronize(dev)
        tf = time.perf_counter()
        ref = Jm @ P[:, :nc]
        torch.cuda.synchronize(dev)
        timings["metric_check"] = {"columns": nc, "max_abs_dB": (B[:, :nc] - ref).abs().max().item(),
                                   "max_abs_B": ref.abs().max().item(),
                                   "fp64_library_gemm_s": time.perf_counter() - tf}
        del ref
    del P, Jm
    torch.cuda.empty_cache()
    rows = B[:keep_rows].cpu().numpy() if keep_rows > 0 else None
    eng.upload_device(B.data_ptr())
    del B
    torch.cuda.empty_cache()
    timings["total_s"] = time.perf_counter() - t0
    eig = timings.pop("metric_eig", None)
    return DeviceDF(eng, nbf, naux, sp, M, Jm_host, ints, timings, rows, eig)


def build_device_B_screened(mol: Molecule, primary: BasisSet, aux: BasisSet, device: int = 0,
                            cutoff: float = DEFAULT_CUTOFF, condition: float = DEFAULT_CONDITION,
                            ints: Integrals | None = None, block: int = 128, upload_rows: int = 256,
                            device_integrals: bool = True, metric_power_on: str = "auto") -> DeviceDF:
    """build_device_B for systems whose dense packed triangle would not fit the device (the
    C100H202 workload: 271 GB dense, 10 % of the pairs significant): (P|mn) is held on the device
    over the Schwarz-significant pairs only (m >= n, DFHelper's sparse tensor), contracted with
    J^-1/2 there, and B is expanded back to packed-triangle rows a block of aux functions at a
    time for the engine's block upload (gdfjk_upload_B_device_block), which keeps only the
    stored tiles.  device_integrals as in build_device_B (the kernels write the significant
    pairs' columns through a column map)."""
    import torch

    dev = torch.device("cuda", device)
    t0 = time.perf_counter()
    ints = ints or Integrals(mol, primary, aux)
    nbf, naux = primary.nbf, aux.nbf
    timings = {}
    ts = time.perf_counter()
    fun_max, shell_max = ints.schwarz()
    sp = prepare_sparsity(fun_max, shell_max, cutoff, naux)
    timings["schwarz_and_sparsity_host_s"] = time.perf_counter() - ts
    r, c = np.tril_indices(nbf)
    sig = np.flatnonzero(sp.pair_mask[r, c])  # packed-triangle columns of the significant pairs
    npair, nsig = r.size, sig.size
    pb_dev = ab_dev = None
    if device_integrals:
        pb_dev, ab_dev = DeviceBasis(primary, device), DeviceBasis(aux, device)
    M, Jm_host, Jm = _metric_and_power(ints, ab_dev, naux, condition, dev, timings, metric_power_on)
    sig_d = torch.from_numpy(sig).to(dev)
    t_ints = t_copy = 0.0
    if device_integrals:
        ta = time.perf_counter()
        col_map = np.full(npair, -1, dtype=np.int64)
        col_map[sig] = np.arange(nsig, dtype=np.int64)
        col_d = torch.from_numpy(col_map).to(dev)
        P = torch.zeros((naux, nsig), dtype=torch.float64, device=dev)
        three_index_device(ab_dev, pb_dev, P.data_ptr(), nsig, shell_mask=sp.shell_mask, col_map_ptr=col_d.data_ptr())
        torch.cuda.synchronize(dev)
        del col_d
        timings["three_index_device_s"] = time.perf_counter() - ta
        pb_dev.close()
        ab_dev.close()
    else:
        P = torch.empty((naux, nsig), dtype=torch.float64, device=dev)
        for p0 in range(0, naux, block):
            p1 = min(naux, p0 + block)
            ta = time.perf_counter()
            A = ints.three_index(shell_mask=sp.shell_mask, p0=p0, p1=p1)
            As = np.ascontiguousarray(A[:, sig])
            del A
            t_ints += time.perf_counter() - ta
            tb = time.perf_counter()
            P[p0:p1] = torch.from_numpy(As).to(dev)
            t_copy += time.perf_counter() - tb
        torch.cuda.synchronize(dev)
        timings.update({"three_index_host_s": t_ints, "three_index_copy_s": t_copy})
    eng = DFJKEngine(nbf, naux, sp.pair_mask, device=device)
    Bs = torch.empty_like(P)
    tg = time.perf_counter()
    eng.metric_contract(Jm.data_ptr(), P.data_ptr(), nsig, Bs.data_ptr())
    t_gemm = time.perf_counter() - tg
    del P, Jm
    torch.cuda.empty_cache()
    tu = time.perf_counter()
    rows = torch.zeros((min(upload_rows, naux), npair), dtype=torch.float64, device=dev)
    for q0 in range(0, naux, upload_rows):
        nq = min(upload_rows, naux - q0)
        rows[:nq].index_copy_(1, sig_d, Bs[q0:q0 + nq])
        torch.cuda.synchronize(dev)
        eng.upload_device_block(rows.data_ptr(), q0, nq)
    del rows, Bs
    torch.cuda.empty_cache()
    t_up = time.perf_counter() - tu
    timings.update({"metric_contraction_device_s": t_gemm, "expand_and_upload_s": t_up, "significant_pairs": int(nsig),
                    "pairs": int(npair), "total_s": time.perf_counter() - t0})
    eig = timings.pop("metric_eig", None)
    return DeviceDF(eng, nbf, naux, sp, M, Jm_host, ints, timings, None, eig)


def slice_pqq(rows: np.ndarray, sp: Sparsity) -> tuple[np.ndarray, Sparsity]:
    """DFHelper's pQq layout (dfhelper.cc:1671-1673) of a block of aux rows given as packed
    triangles, with the sparsity tables re-indexed for that many rows."""
    nq, nbf = rows.shape[0], sp.nbf
    s2 = prepare_sparsity(sp.pair_mask.astype(np.float64), sp.shell_mask.astype(np.float64), 1.0, nq)
    out = np.zeros(int(s2.big_skips[nbf]))
    for m in range(nbf):
        sig = np.flatnonzero(sp.pair_mask[m])
        if sig.size == 0:
            continue
        hi, lo = np.maximum(sig, m), np.minimum(sig, m)
        out[s2.big_skips[m]: s2.big_skips[m + 1]] = rows[:, hi * (hi + 1) // 2 + lo].reshape(-1)
    return out, s2
