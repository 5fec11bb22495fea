"""B = J^-1/2 (P|mn) built on the device for large systems (the caller's initialisation).

This is psi4's ``DFHelper::prepare_AO_core`` (psi4/src/psi4/lib3index/dfhelper.cc:514-588)
arranged for one GB300: the raw 3-index integrals (P|mn) come from the host integral
provider in blocks of aux rows (``compute_sparse_pQq_blocking_p_symm``, dfhelper.cc:1284-1347)
and are copied into one device array; the metric contraction (``contract_metric_AO_core_symm``,
dfhelper.cc:1653-1678) runs on the tensor cores to FP64 accuracy
(``gdfjk_metric_contract_device``); B is then relaid into the engine's tiles
(``gdfjk_upload_B_device``).  Screening and the metric power are the host restatements of
``dfhelper.py`` (prepare_sparsity, Matrix::power).

torch supplies the device arrays (plumbing); every computation on them is the engine's.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np

from .basis import BasisSet
from .dfhelper import DEFAULT_CONDITION, DEFAULT_CUTOFF, Sparsity, metric_power, prepare_sparsity
from .ints import Integrals
from .jk import DFJKEngine
from .molecule import Molecule


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


def build_device_B(mol: Molecule, primary: BasisSet, aux: BasisSet, device: int = 0, cutoff: float = DEFAULT_CUTOFF,
                   condition: float = DEFAULT_CONDITION, ints: Integrals | None = None, block: int = 128,
                   keep_rows: int = 0, check_columns: int = 0) -> DeviceDF:
    """Build B on the device and upload it into a new engine.  `keep_rows` > 0 also returns a
    host copy of B's first rows (for checks against a CPU restatement); `check_columns` > 0
    compares that many columns of the tensor-core metric contraction with the FP64 library
    GEMM and records the largest difference in ``timings``."""
    import torch

    dev = torch.device("cuda", device)
    t0 = time.perf_counter()
    ints = ints or Integrals(mol, primary, aux)
    nbf, naux = primary.nbf, aux.nbf
    fun_max, shell_max = ints.schwarz()
    sp = prepare_sparsity(fun_max, shell_max, cutoff, naux)
    M = ints.metric()
    Jm_host = metric_power(M, -0.5, condition)
    Jm = torch.from_numpy(Jm_host).to(dev).contiguous()
    r, c = np.tril_indices(nbf)
    keep = torch.from_numpy(sp.pair_mask[r, c].astype(np.float64)).to(dev)
    npair = keep.numel()
    P = torch.empty((naux, npair), dtype=torch.float64, device=dev)
    t_ints = t_copy = 0.0
    for p0 in range(0, naux, block):
        p1 = min(naux, p0 + block)
        ta = time.perf_counter()
        A = ints.three_index(shell_mask=sp.shell_mask, p0=p0, p1=p1)
        t_ints += time.perf_counter() - ta
        tb = time.perf_counter()
        P[p0:p1] = torch.from_numpy(A).to(dev) * keep  # screened pairs are absent from psi4's tensor
        torch.cuda.synchronize(dev)
        t_copy += time.perf_counter() - tb
    del keep
    eng = DFJKEngine(nbf, naux, sp.pair_mask, device=device)
    B = torch.empty((naux, npair), dtype=torch.float64, device=dev)
    torch.cuda.synchronize(dev)
    tg = time.perf_counter()
    eng.metric_contract(Jm.data_ptr(), P.data_ptr(), npair, B.data_ptr())
    t_gemm = time.perf_counter() - tg
    timings = {"three_index_host_s": t_ints, "three_index_copy_s": t_copy, "metric_contraction_device_s": t_gemm}
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
    return DeviceDF(eng, nbf, naux, sp, M, Jm_host, ints, timings, rows)


def build_device_B_screened(mol: Molecule, primary: BasisSet, aux: BasisSet, device: int = 0,
                            cutoff: float = DEFAULT_CUTOFF, condition: float = DEFAULT_CONDITION,
                            ints: Integrals | None = None, block: int = 128, upload_rows: int = 256) -> DeviceDF:
    """build_device_B for systems whose dense packed triangle would not fit the device (the
    C100H202 workload: 271 GB dense, 10 % of the pairs significant): (P|mn) is held on the device
    over the Schwarz-significant pairs only (m >= n, DFHelper's sparse tensor), contracted with
    J^-1/2 there, and B is expanded back to packed-triangle rows a block of aux functions at a
    time for the engine's block upload (gdfjk_upload_B_device_block), which keeps only the
    stored tiles."""
    import torch

    dev = torch.device("cuda", device)
    t0 = time.perf_counter()
    ints = ints or Integrals(mol, primary, aux)
    nbf, naux = primary.nbf, aux.nbf
    fun_max, shell_max = ints.schwarz()
    sp = prepare_sparsity(fun_max, shell_max, cutoff, naux)
    r, c = np.tril_indices(nbf)
    sig = np.flatnonzero(sp.pair_mask[r, c])  # packed-triangle columns of the significant pairs
    npair, nsig = r.size, sig.size
    M = ints.metric()
    tm = time.perf_counter()
    Jm_host = metric_power(M, -0.5, condition)
    t_metric = time.perf_counter() - tm
    sig_d = torch.from_numpy(sig).to(dev)
    P = torch.empty((naux, nsig), dtype=torch.float64, device=dev)
    t_ints = t_copy = 0.0
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
    eng = DFJKEngine(nbf, naux, sp.pair_mask, device=device)
    Jm = torch.from_numpy(Jm_host).to(dev)
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
    timings = {"three_index_host_s": t_ints, "three_index_copy_s": t_copy, "metric_power_host_s": t_metric,
               "metric_contraction_device_s": t_gemm, "expand_and_upload_s": t_up, "significant_pairs": int(nsig),
               "pairs": int(npair), "total_s": time.perf_counter() - t0}
    return DeviceDF(eng, nbf, naux, sp, M, Jm_host, ints, timings, None)


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
