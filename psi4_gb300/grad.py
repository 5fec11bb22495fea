"""RHF nuclear gradient with the density-fitted two-electron part from the GB300 engine.

The engine's backward (``gdfjk_backward``) returns Gamma = dE/dB in B-space
(B = M^-1/2 A, A = raw (P|mn), M = (P|Q)), which is mapped to the raw-integral densities
psi4's DFJKGrad contracts with derivative integrals (psi4/src/psi4/scfgrad/jk_grad.cc:175-293,
build_AB_x_terms :834-867, build_Amn_x_terms :868-1245) — with an engine, on the device:
A from the engine's integral kernels, the two metric products on the tensor cores / the
FP64 library, and both derivative-integral contractions in the engine's derivative kernels
(gdfjk_three_index_grad_device, gdfjk_metric_grad_device); without one, on the host:

    3-index density  G3 = dE/dA = M^-1/2 Gamma
    2-index density  G2 = dE/dM = Frechet derivative of M -> M^-1/2 applied to
                     W = Gamma A^T (eigenbasis form, same eigenvalue truncation as the
                     forward Matrix::power, psi4/src/psi4/libmints/matrix.cc:2370-2415)

and assembles (scf_grad.cc:196-296, restricted case, alpha densities D and W):

    dE/dx = E_nuc^x + 2 D.(T^x + V^x) - 2 W.S^x + G3.(A|mn)^x + G2.(P|Q)^x
"""
from __future__ import annotations

import numpy as np


def metric_power_frechet(M, W, power=-0.5, condition=1e-10):
    """dE/dM given dE/dF = W for F = M^power with psi4's eigenvalue truncation."""
    w, V = np.linalg.eigh(M)
    max_a = max(abs(w[-1]), abs(w[0]))
    keep = np.abs(w) >= condition * max_a if power < 0 else np.ones_like(w, dtype=bool)
    f = np.where(keep, np.abs(w) ** power, 0.0)
    fp = np.where(keep, power * np.abs(w) ** (power - 1.0), 0.0)
    dl = w[:, None] - w[None, :]
    with np.errstate(divide="ignore", invalid="ignore"):
        Lm = (f[:, None] - f[None, :]) / dl
    same = np.abs(dl) <= 1e-14 * np.maximum(1.0, np.abs(w[:, None]))
    Lm = np.where(same, 0.5 * (fp[:, None] + fp[None, :]), Lm)
    Ws = 0.5 * (W + W.T)
    return V @ (Lm * (V.T @ Ws @ V)) @ V.T


def metric_power_frechet_device(Md, Wd, power=-0.5, condition=1e-10, eig=None):
    """metric_power_frechet on device arrays (the library's FP64 eigensolver and GEMMs), for
    large fitting sets; same truncation and divided differences.  eig: the metric's (w, V)
    from its power at initialisation (the eigensolver is then skipped).  All four products
    stay FP64: the divided differences reach lambda_min^-3/2 (~1e13 with the kept eigenvalues)
    and cancel in the back-rotation, so a digit product, whose error is relative to row and
    column maxima, is not usable here (it gave errors of 1e8 on (H2O)_8)."""
    import torch

    w, V = eig if eig is not None else torch.linalg.eigh(Md)
    max_a = torch.maximum(w[-1].abs(), w[0].abs())
    aw = w.abs()
    keep = aw >= condition * max_a if power < 0 else torch.ones_like(w, dtype=torch.bool)
    safe = torch.where(keep, aw, torch.ones_like(aw))
    f = torch.where(keep, safe ** power, torch.zeros_like(w))
    fp = torch.where(keep, power * safe ** (power - 1.0), torch.zeros_like(w))
    dl = w[:, None] - w[None, :]
    same = dl.abs() <= 1e-14 * torch.clamp(w[:, None].abs(), min=1.0)
    Lm = torch.where(same, 0.5 * (fp[:, None] + fp[None, :]), (f[:, None] - f[None, :]) / torch.where(same, torch.ones_like(dl), dl))
    Ws = 0.5 * (Wd + Wd.T)
    return V @ (Lm * (V.T @ Ws @ V)) @ V.T


def two_electron_gradient_screened(engine, ints, sp, metric, Jmhalf, C, timings=None, batch_q=0, callback=None,
                                   metric_eig=None):
    """The two-electron gradient with every naux x pairs array kept over the significant pairs
    only (the layout of device_init.build_device_B_screened), for systems whose dense triangle
    would not fit (C100H202): Gamma = dE/dB from the engine's batched backward with (Q|mi)
    recomputed (gdfjk_backward_gamma_device), G3 = M^-1/2 Gamma and W = Gamma A^T on the
    tensor cores (FP64-accurate digit products; W's digit error moved the (H2O)_16 gradient by
    5e-8 Eh/bohr), A from the integral kernels, the Frechet derivative of M^-1/2 on the device,
    and the derivative contractions in the derivative kernels.  C: occupied orbitals (host);
    the tensor-core forms' copies of B are released first (rebuilt by the next build).
    callback() is called after each large piece (memory sampling); metric_eig: the metric's
    eigenpairs on the device from its power at initialisation (DeviceDF.metric_eig)."""
    import time

    import torch

    from .device_init import DeviceBasis, metric_grad_device, three_index_device, three_index_grad_device

    dev = torch.device("cuda", engine.device)
    nbf, nocc = C.shape
    naux = metric.shape[0]
    natom = ints.mol.natom
    tm = {}
    t = time.perf_counter()
    r, c = np.tril_indices(nbf)
    sig = np.flatnonzero(sp.pair_mask[r, c])
    nsig = sig.size
    col_map = np.full(r.size, -1, dtype=np.int64)
    col_map[sig] = np.arange(nsig, dtype=np.int64)
    col_d = torch.from_numpy(col_map).to(dev)
    engine.trim()
    Cd = torch.from_numpy(np.ascontiguousarray(C)).to(dev)
    D = Cd @ Cd.T
    gJ, gK = 2.0 * D, -D
    G = torch.empty((naux, nsig), dtype=torch.float64, device=dev)
    engine.backward_gamma_device(Cd.data_ptr(), nocc, nocc, gJ.data_ptr(), gK.data_ptr(), G.data_ptr(), nsig,
                                 col_map_ptr=col_d.data_ptr(), batch_q=batch_q)
    del D, gJ, gK
    if callback:
        callback()
    t1 = time.perf_counter()
    Jm = torch.from_numpy(np.ascontiguousarray(Jmhalf)).to(dev)
    G3 = torch.empty_like(G)
    engine.gemm(Jm.data_ptr(), naux, G.data_ptr(), nsig, G3.data_ptr(), nsig, naux, nsig, naux)
    del Jm
    t2 = time.perf_counter()
    pd, ad = DeviceBasis(ints.primary, engine.device), DeviceBasis(ints.aux, engine.device)
    A = torch.zeros_like(G)
    three_index_device(ad, pd, A.data_ptr(), nsig, shell_mask=sp.shell_mask, col_map_ptr=col_d.data_ptr())
    if callback:
        callback()
    t3 = time.perf_counter()
    # W = Gamma A^T over chunks of the pairs (the digit copies of both operands stay ~8 GB)
    W = torch.empty((naux, naux), dtype=torch.float64, device=dev)
    kc = max(1024, int(8e9 / (16.0 * naux)) // 1024 * 1024)
    for k0 in range(0, nsig, kc):
        k1 = min(nsig, k0 + kc)
        engine.gemm(G.data_ptr() + 8 * k0, nsig, A.data_ptr() + 8 * k0, nsig, W.data_ptr(), naux, naux, naux, k1 - k0,
                    transb=True, accumulate=k0 > 0)
    del A, G
    torch.cuda.empty_cache()
    t4 = time.perf_counter()
    Md = torch.from_numpy(np.ascontiguousarray(metric)).to(dev)
    G2 = metric_power_frechet_device(Md, W, eig=metric_eig)
    del Md, W
    torch.cuda.synchronize(dev)
    t5 = time.perf_counter()
    g = torch.zeros((natom, 3), dtype=torch.float64, device=dev)
    three_index_grad_device(ad, pd, G3.data_ptr(), nsig, natom, g.data_ptr(), shell_mask=sp.shell_mask,
                            col_map_ptr=col_d.data_ptr())
    t6 = time.perf_counter()
    metric_grad_device(ad, G2.data_ptr(), naux, natom, g.data_ptr())
    out = g.cpu().numpy()
    t7 = time.perf_counter()
    del G3, G2, col_d
    pd.close()
    ad.close()
    torch.cuda.empty_cache()
    if timings is not None:
        timings.update({"backward_gamma_s": t1 - t, "metric_product_G3_s": t2 - t1, "three_index_s": t3 - t2,
                        "metric_product_W_s": t4 - t3, "metric_frechet_device_s": t5 - t4,
                        "three_index_derivative_contraction_s": t6 - t5, "metric_derivative_contraction_s": t7 - t6,
                        "significant_pairs": int(nsig)})
    return out


def _two_electron_gradient_device(engine, ints, df, Gamma, timings):
    """The device path: A = (P|mn) from the integral kernels (screened function pairs zero, as
    in the DF tensor), G3 = M^-1/2 Gamma on the tensor cores, W = Gamma A^T in FP64, the
    Frechet derivative of M^-1/2 on the host, and both derivative contractions on the device."""
    import time

    import torch

    from .device_init import DeviceBasis, metric_grad_device, three_index_device, three_index_grad_device

    dev = torch.device("cuda", engine.device)
    sp = df.sparsity
    naux, npair = Gamma.shape
    natom = ints.mol.natom
    t = time.perf_counter()
    pd, ad = DeviceBasis(ints.primary, engine.device), DeviceBasis(ints.aux, engine.device)
    A = torch.zeros((naux, npair), dtype=torch.float64, device=dev)
    three_index_device(ad, pd, A.data_ptr(), npair, shell_mask=sp.shell_mask)
    r, c = np.tril_indices(df.nbf)
    A *= torch.from_numpy(sp.pair_mask[r, c].astype(np.float64)).to(dev)
    torch.cuda.synchronize(dev)
    t1 = time.perf_counter()
    Gd = torch.from_numpy(np.ascontiguousarray(Gamma)).to(dev)
    Jm = torch.from_numpy(np.ascontiguousarray(df.Jmhalf)).to(dev)
    G3 = torch.empty_like(Gd)
    engine.gemm(Jm.data_ptr(), naux, Gd.data_ptr(), npair, G3.data_ptr(), npair, naux, npair, naux)
    W = (Gd @ A.T).cpu().numpy()
    del A, Gd, Jm
    t2 = time.perf_counter()
    G2 = metric_power_frechet(df.metric, W)
    t3 = time.perf_counter()
    g = torch.zeros((natom, 3), dtype=torch.float64, device=dev)
    three_index_grad_device(ad, pd, G3.data_ptr(), npair, natom, g.data_ptr(), shell_mask=sp.shell_mask)
    t4 = time.perf_counter()
    G2d = torch.from_numpy(np.ascontiguousarray(G2)).to(dev)
    metric_grad_device(ad, G2d.data_ptr(), naux, natom, g.data_ptr())
    out = g.cpu().numpy()
    t5 = time.perf_counter()
    pd.close()
    ad.close()
    if timings is not None:
        timings.update({"three_index_s": t1 - t, "metric_products_s": t2 - t1, "metric_frechet_s": t3 - t2,
                        "three_index_derivative_contraction_s": t4 - t3, "metric_derivative_contraction_s": t5 - t4,
                        "metric_products_on": "tensor cores (G3) and the FP64 library (W)",
                        "integrals_and_derivative_contractions_on": "device"})
    return out


def two_electron_gradient(ints, df, Gamma, A_raw=None, engine=None, timings=None):
    """Contract Gamma (dE/dB, packed) with derivative integrals through B = M^-1/2 A.  With an
    engine everything but the Frechet derivative of M^-1/2 runs on its device (integrals,
    metric products, derivative contractions); `timings` (a dict) receives the seconds of each
    piece."""
    import time

    if engine is not None:
        return _two_electron_gradient_device(engine, ints, df, Gamma, timings)
    t = time.perf_counter()
    if A_raw is None:
        A_raw = ints.three_index(shell_mask=df.sparsity.shell_mask)
        r, c = np.tril_indices(df.nbf)
        A_raw[:, ~df.sparsity.pair_mask[r, c]] = 0.0
    t1 = time.perf_counter()
    G3 = df.Jmhalf @ Gamma
    W = Gamma @ A_raw.T
    t2 = time.perf_counter()
    G2 = metric_power_frechet(df.metric, W)
    t3 = time.perf_counter()
    g3 = ints.three_index_grad(G3, shell_mask=df.sparsity.shell_mask)
    t4 = time.perf_counter()
    g2 = ints.metric_grad(G2)
    t5 = time.perf_counter()
    if timings is not None:
        timings.update({"three_index_s": t1 - t, "metric_products_s": t2 - t1, "metric_frechet_s": t3 - t2,
                        "three_index_derivative_contraction_s": t4 - t3, "metric_derivative_contraction_s": t5 - t4,
                        "metric_products_on": "host"})
    return g3 + g2


def one_electron_gradient(mol, ints, scf):
    """E_nuc^x + 2 D.(T^x + V^x) - 2 W.S^x (host provider), D and W from the occupied orbitals."""
    nocc = scf.nocc
    C = scf.C[:, :nocc]
    eps = scf.eps[:nocc]
    D = C @ C.T
    W = (C * eps) @ C.T
    g = mol.nuclear_repulsion_grad()
    g += 2.0 * ints.kinetic_grad(D)
    g += 2.0 * ints.potential_grad(D)
    g -= 2.0 * ints.overlap_grad(W)
    return g


def one_electron_gradient_device(mol, ints, scf, device=0):
    """one_electron_gradient with the nuclear-attraction derivatives on the device
    (gdfjk_potential_grad_device; O(natom nbf^2) integrals, the expensive part at C100H202);
    the kinetic and overlap derivatives and E_nuc stay on the host."""
    import torch

    from .device_init import DeviceBasis, potential_grad_device

    nocc = scf.nocc
    C = scf.C[:, :nocc]
    eps = scf.eps[:nocc]
    D = C @ C.T
    W = (C * eps) @ C.T
    g = mol.nuclear_repulsion_grad()
    g += 2.0 * ints.kinetic_grad(D)
    g -= 2.0 * ints.overlap_grad(W)
    nbf = D.shape[0]
    r, c = np.tril_indices(nbf)
    Dp = np.where(r == c, 1.0, 2.0) * D[r, c]  # sum over m >= n with both (mn) and (nm)
    dev = torch.device("cuda", device)
    Dd = torch.from_numpy(np.ascontiguousarray(Dp)).to(dev)
    gd = torch.zeros((mol.natom, 3), dtype=torch.float64, device=dev)
    pd = DeviceBasis(ints.primary, device)
    potential_grad_device(pd, Dd.data_ptr(), mol, gd.data_ptr())
    pd.close()
    return g + 2.0 * gd.cpu().numpy()


def rhf_gradient(mol, ints, df, scf, Gamma, engine=None, timings=None):
    """Total RHF gradient (natom x 3, Eh/bohr) from a converged SCF and the engine's Gamma
    for gJ = dE/dJ = 2D, gK = dE/dK = -D: with `engine` the two-electron part on its device,
    else on the host (the one-electron terms on the host either way)."""
    return one_electron_gradient(mol, ints, scf) + two_electron_gradient(ints, df, Gamma, engine=engine,
                                                                         timings=timings)
