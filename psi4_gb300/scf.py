"""Restricted Hartree-Fock driver around a psi4.core.JK-shaped object.

This is the caller side of the DF-JK path: psi4's ``scf_iterate``
(psi4/driver/procrouting/scf_proc/scf_iterator.py:264-609) with ``RHF::form_G`` /
``form_F`` / ``compute_E`` / ``form_C`` / ``form_D`` (psi4/src/psi4/libscf_solver/rhf.cc:
187-370, hf.cc:1330).  Each iteration pushes the occupied orbitals into the JK object,
calls ``compute()`` and reads ``J()[0]``/``K()[0]``:

    G = 2J - K,  F = H + G,  E = E_nuc + 2 tr(D H) + 2 tr(D J) - tr(D K)   (alpha D = C_occ C_occ^T)

DIIS (Pulay, on the orthogonalised FDS - SDF, up to 10 vectors) and the diagonalisation
stay FP64 on the host.  Convergence as ``_converged`` (scf_iterator.py:929):
|dE| < e_conv and RMS orbital gradient < d_conv.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field

import numpy as np


class SCFConvergenceError(RuntimeError):
    """Raised when the SCF does not converge in maxiter (scf_iterator.py:608-609)."""

    def __init__(self, msg, result):
        super().__init__(msg)
        self.result = result


@dataclass
class SCFResult:
    energy: float
    energies: list
    iterations: int
    converged: bool
    C: np.ndarray
    eps: np.ndarray
    D: np.ndarray
    F: np.ndarray
    J: np.ndarray
    K: np.ndarray
    nocc: int
    timings: dict = field(default_factory=dict)
    log: list = field(default_factory=list)
    orbitals: list = field(default_factory=list)


def orthogonalizer(S, tol=1e-7):
    """Symmetric S^-1/2, or canonical when the smallest eigenvalue is below S_TOLERANCE
    (psi4 default 1e-7)."""
    w, V = np.linalg.eigh(S)
    if w.min() >= tol:
        return (V / np.sqrt(w)) @ V.T
    keep = w >= tol
    return V[:, keep] / np.sqrt(w[keep])


def _gradient(F, Cocc, S, X):
    """X^T (F D S - S D F) X for D = Cocc Cocc^T without forming F D S: with A = X^T F Cocc and
    B = X^T S Cocc it is A B^T - B A^T (F, S symmetric), O(nbf^2 nocc) instead of O(nbf^3)."""
    A = X.T @ (F @ Cocc)
    B = X.T @ (S @ Cocc)
    return A @ B.T - B @ A.T


class DIIS:
    """Pulay DIIS over at most `max_vec` (F, error) pairs; the error inner products are kept
    between iterations, so adding a vector costs one product per stored vector."""

    def __init__(self, max_vec=10):
        self.max_vec = max_vec
        self.F, self.E = [], []
        self.G = np.zeros((0, 0))

    def add(self, F, err):
        if len(self.F) == self.max_vec:
            self.F.pop(0)
            self.E.pop(0)
            self.G = self.G[1:, 1:]
        self.F.append(F.copy())
        self.E.append(err.copy())
        n = len(self.E)
        G = np.zeros((n, n))
        G[:n - 1, :n - 1] = self.G
        for i in range(n):
            G[i, n - 1] = G[n - 1, i] = float(np.vdot(self.E[i], self.E[n - 1]))
        self.G = G

    def extrapolate(self):
        n = len(self.F)
        B = -np.ones((n + 1, n + 1))
        B[n, n] = 0.0
        B[:n, :n] = self.G
        rhs = np.zeros(n + 1)
        rhs[n] = -1.0
        # scale for conditioning
        d = np.abs(np.diag(B[:n, :n])).max()
        if d > 0:
            B[:n, :n] /= d
        try:
            c = np.linalg.solve(B, rhs)[:n]
        except np.linalg.LinAlgError:
            c = np.linalg.lstsq(B, rhs, rcond=None)[0][:n]
        return sum(ci * Fi for ci, Fi in zip(c, self.F))


class PrecisionSchedule:
    """The precision form's build schedule for a GpuDFJK.

    1. split-BF16 incremental K builds (over dD) from the guess;
    2. once the RMS orbital gradient drops below anchor_d: one FP64 full build that becomes
       the base of the following increments (their errors then scale with the now small dD);
    3. split-BF16 increments again until |dE| < switch_e and RMS gradient < switch_d;
    4. FP64 full rebuilds to convergence.  Convergence is only accepted on an FP64 build that
       follows another FP64 build, so the final two Fock builds are full FP64 rebuilds and
       the converged energy is an FP64 energy."""

    def __init__(self, anchor_d=1e-3, switch_e=1e-8, switch_d=1e-6, max_mixed=60, report_fp64=None,
                 fp64_precision="fp64"):
        self.anchor_d, self.switch_e, self.switch_d, self.max_mixed = anchor_d, switch_e, switch_d, max_mixed
        self.fp64_precision = fp64_precision  # "fp64" or "fp64-emulated" for the FP64 builds
        self.report_fp64 = report_fp64  # optional JK (FP64) to measure each mixed energy's error
        self.mode = "mixed"
        self.anchored = anchor_d is None
        self.n_mixed = 0
        self.n_fp64 = 0
        self.n_anchor = 0
        self.fp64_streak = 0

    def before(self, jk):
        if self.mode == "anchor":
            jk.set_precision(self.fp64_precision)
            jk.set_incremental(True)
        else:
            jk.set_precision("mixed" if self.mode == "mixed" else self.fp64_precision)
            jk.set_incremental(self.mode == "mixed")

    def after(self, dE, dnorm):
        if self.mode == "mixed":
            self.n_mixed += 1
            self.fp64_streak = 0
            if not self.anchored and dnorm < self.anchor_d:
                self.mode = "anchor"
            elif (abs(dE) < self.switch_e and dnorm < self.switch_d) or self.n_mixed >= self.max_mixed:
                self.mode = "fp64"
        elif self.mode == "anchor":
            self.n_anchor += 1
            self.n_fp64 += 1
            self.anchored = True
            self.mode = "mixed"
        else:
            self.n_fp64 += 1
            self.fp64_streak += 1

    def may_converge(self):
        return self.fp64_streak >= 2


def sad_guess(mol, basis: str, maxiter: int = 60, conv: float = 1e-8) -> np.ndarray:
    """psi4's default SCF guess, superposition of atomic densities (libscf_solver/sad.cc): one
    spin-averaged SCF per element in its own basis (fractional occupation of the open shell,
    spread evenly over its degenerate orbitals; J and K from the atom's density-fitted
    integrals), the molecular alpha density the block-diagonal sum of the atomic ones over
    psi4's atom-by-atom function order.  Returns a factor Cs (nbf x k) with Cs Cs^T that
    density (each atomic natural orbital scaled by the square root of half its occupation),
    ready to be pushed into a JK object like occupied orbitals."""
    from .basis import BasisSet
    from .dfhelper import build_df_tensor
    from .ints import Integrals
    from .molecule import Molecule

    factors = {}
    for sym in dict.fromkeys(mol.symbols):
        amol = Molecule([sym], np.zeros((1, 3)))
        pb = BasisSet.build(amol, basis)
        ab = BasisSet.fitting_for(amol, pb)
        ints = Integrals(amol, pb, ab)
        B = build_df_tensor(amol, pb, ab, ints=ints).dense()  # (naux, n, n), a few hundred KB
        Ha, Sa = core_hamiltonian(ints), ints.overlap()
        Xa = orthogonalizer(Sa)
        nel = float(amol.nelectron)
        D = np.zeros_like(Ha)
        Dold = None
        for _ in range(maxiter):
            J = np.einsum("qmn,q->mn", B, np.einsum("qls,ls->q", B, D))
            K = np.einsum("qml,ls,qsn->mn", B, D, B)
            F = Ha + J - 0.5 * K  # spin-averaged closed-shell form of the total density D
            eps, Cp = np.linalg.eigh(Xa.T @ F @ Xa)
            Ca = Xa @ Cp
            occ = np.zeros(eps.size)
            left, i = nel, 0
            while left > 1e-12 and i < eps.size:
                deg = np.flatnonzero(np.abs(eps - eps[i]) < 1e-4)
                deg = deg[deg >= i]
                take = min(left, 2.0 * deg.size)
                occ[deg] = take / deg.size
                left -= take
                i = deg[-1] + 1
            Dn = (Ca * occ) @ Ca.T
            D = Dn if Dold is None else 0.5 * (Dn + Dold)
            if Dold is not None and np.abs(D - Dold).max() < conv:
                break
            Dold = D
        keep = occ > 0
        factors[sym] = Ca[:, keep] * np.sqrt(occ[keep] / 2.0)  # alpha density = D / 2
    blocks, nbf_atoms = [], []
    for sym in mol.symbols:
        blocks.append(factors[sym])
        nbf_atoms.append(factors[sym].shape[0])
    nbf, k = sum(nbf_atoms), sum(b.shape[1] for b in blocks)
    Cs = np.zeros((nbf, k))
    r = c = 0
    for blk in blocks:
        Cs[r:r + blk.shape[0], c:c + blk.shape[1]] = blk
        r += blk.shape[0]
        c += blk.shape[1]
    return Cs


def rhf(jk, H, S, nocc, e_nuc, e_conv=1e-10, d_conv=1e-8, maxiter=100, guess_C=None, diis_start=1,
        fail_on_maxiter=True, callback=None, verbose=False, schedule: PrecisionSchedule | None = None,
        record_orbitals=False, guess_density_factor=None) -> SCFResult:
    """Run RHF with a JK object exposing C_clear/C_left_add/compute/J/K.  With a
    PrecisionSchedule the JK switches between the mixed and FP64 forms per iteration.
    `record_orbitals` keeps every iteration's occupied orbitals in ``result.orbitals`` (for
    evaluating afterwards the FP64 energy at each iterate: `energy_errors_vs_fp64`).
    `guess_density_factor` (e.g. `sad_guess`): the first Fock build is made from that density
    instead of the core guess's orbitals, as psi4 does with its SAD guess."""
    X = orthogonalizer(S)
    t0 = time.perf_counter()
    if guess_density_factor is not None:
        C = np.ascontiguousarray(guess_density_factor)
        eps = np.zeros(C.shape[1])
    elif guess_C is None:
        # core guess
        eps, Cp = np.linalg.eigh(X.T @ H @ X)
        C = X @ Cp
    else:
        C = guess_C
        eps = np.zeros(C.shape[1])
    diis = DIIS()
    E_old = 0.0
    energies = []
    log = []
    t_jk = 0.0
    converged = False
    it = 0
    F = J = K = D = None
    orbitals = []
    for it in range(1, maxiter + 1):
        Cocc = np.ascontiguousarray(C if (it == 1 and guess_density_factor is not None) else C[:, :nocc])
        if record_orbitals:
            orbitals.append(Cocc)
        D = Cocc @ Cocc.T
        jk.C_clear()
        jk.C_left_add(Cocc)
        mode = None
        if schedule is not None:
            schedule.before(jk)
            mode = schedule.mode
        tj = time.perf_counter()
        jk.compute()
        t_jk += time.perf_counter() - tj
        J = np.asarray(jk.J()[0])
        K = np.asarray(jk.K()[0])
        F = H + 2.0 * J - K
        E = e_nuc + 2.0 * np.vdot(D, H) + 2.0 * np.vdot(D, J) - np.vdot(D, K)
        energies.append(float(E))
        grad = _gradient(F, Cocc, S, X)  # X^T (FDS - SDF) X
        dnorm = float(np.sqrt(np.mean(grad * grad)))
        dE = E - E_old
        entry = {"iter": it, "energy": float(E), "dE": float(dE), "dnorm": dnorm}
        if mode is not None:
            entry["precision"] = mode
            if mode in ("mixed", "anchor") and schedule.report_fp64 is not None:
                ref = schedule.report_fp64
                ref.C_clear()
                ref.C_left_add(Cocc)
                ref.compute()
                Jr, Kr = np.asarray(ref.J()[0]), np.asarray(ref.K()[0])
                Er = e_nuc + 2.0 * np.vdot(D, H) + 2.0 * np.vdot(D, Jr) - np.vdot(D, Kr)
                entry["energy_error_vs_fp64"] = float(E - Er)
        log.append(entry)
        if verbose:
            print(f"  @RHF iter {it:3d}: {E:20.14f} {dE: .3e} {dnorm: .3e} {mode or ''}")
        if callback is not None:
            callback(it, E, dE, dnorm, D)
        if schedule is not None:
            schedule.after(dE, dnorm)
        if abs(dE) < e_conv and dnorm < d_conv and (schedule is None or schedule.may_converge()):
            converged = True
            break
        E_old = E
        if it >= diis_start:
            diis.add(F, grad)
            Fd = diis.extrapolate() if len(diis.F) >= 2 else F
        else:
            Fd = F
        eps, Cp = np.linalg.eigh(X.T @ Fd @ X)
        C = X @ Cp
    res = SCFResult(energies[-1], energies, it, converged, C, eps, D, F, J, K, nocc,
                    {"total_s": time.perf_counter() - t0, "jk_s": t_jk}, log, orbitals)
    if not converged and fail_on_maxiter:
        raise SCFConvergenceError(f"Could not converge SCF iterations in {maxiter} iterations.", res)
    return res


def rhf_energy(jk, Cocc, H, e_nuc):
    """E = E_nuc + 2 tr(D H) + 2 tr(D J) - tr(D K) at the occupied orbitals Cocc, with J and
    K from one build of `jk` in whatever form it is set to (RHF::compute_E, rhf.cc:308-370)."""
    jk.C_clear()
    jk.C_left_add(np.ascontiguousarray(Cocc))
    jk.compute()
    J, K = np.asarray(jk.J()[0]), np.asarray(jk.K()[0])
    D = Cocc @ Cocc.T
    return float(e_nuc + 2.0 * np.vdot(D, H) + 2.0 * np.vdot(D, J) - np.vdot(D, K))


def energy_errors_vs_fp64(res: SCFResult, fp64_jk, H, e_nuc):
    """For an SCF run with recorded orbitals: each iteration's energy minus the FP64 energy
    at the same orbitals (one FP64 build of `fp64_jk` per iteration), written into
    ``res.log[i]["energy_error_vs_fp64"]``; returns the list of errors."""
    errs = []
    for entry, Cocc in zip(res.log, res.orbitals):
        e = entry["energy"] - rhf_energy(fp64_jk, Cocc, H, e_nuc)
        entry["energy_error_vs_fp64"] = e
        errs.append(e)
    return errs


def core_hamiltonian(ints):
    return ints.kinetic() + ints.potential()


@dataclass
class UHFResult:
    energy: float
    energies: list
    iterations: int
    converged: bool
    Ca: np.ndarray
    Cb: np.ndarray
    Da: np.ndarray
    Db: np.ndarray
    nalpha: int
    nbeta: int
    timings: dict = field(default_factory=dict)
    log: list = field(default_factory=list)


def uhf(jk, H, S, nalpha, nbeta, e_nuc, e_conv=1e-10, d_conv=1e-8, maxiter=100, diis_start=1, fail_on_maxiter=True,
        verbose=False) -> UHFResult:
    """Unrestricted HF through the same JK object: psi4's ``UHF::form_G`` pushes the alpha and
    beta occupied orbitals as two lr-symmetric densities and reads J[0] + J[1], K[0], K[1]
    (psi4/src/psi4/libscf_solver/uhf.cc:184-230); ``compute_E`` (uhf.cc:361-410):

        E = E_nuc + sum_s tr(D_s H) + 1/2 sum_s tr(D_s J) - 1/2 sum_s tr(D_s K_s),  F_s = H + J - K_s

    Core guess, DIIS on the stacked alpha/beta orbital gradients, convergence as ``rhf``."""
    X = orthogonalizer(S)
    t0 = time.perf_counter()
    eps, Cp = np.linalg.eigh(X.T @ H @ X)
    Ca = Cb = X @ Cp
    diis = DIIS()
    E_old = 0.0
    energies, log = [], []
    t_jk = 0.0
    converged = False
    it = 0
    Da = Db = None
    for it in range(1, maxiter + 1):
        Ca_occ = np.ascontiguousarray(Ca[:, :nalpha])
        Cb_occ = np.ascontiguousarray(Cb[:, :nbeta])
        Da, Db = Ca_occ @ Ca_occ.T, Cb_occ @ Cb_occ.T
        jk.C_clear()
        jk.C_left_add(Ca_occ)
        jk.C_left_add(Cb_occ)
        tj = time.perf_counter()
        jk.compute()
        t_jk += time.perf_counter() - tj
        Js, Ks = jk.J(), jk.K()
        J = np.asarray(Js[0]) + np.asarray(Js[1])
        Ka, Kb = np.asarray(Ks[0]), np.asarray(Ks[1])
        Fa, Fb = H + J - Ka, H + J - Kb
        E = (e_nuc + np.vdot(Da + Db, H) + 0.5 * np.vdot(Da + Db, J) - 0.5 * np.vdot(Da, Ka)
             - 0.5 * np.vdot(Db, Kb))
        energies.append(float(E))
        ga = _gradient(Fa, Ca_occ, S, X)
        gb = _gradient(Fb, Cb_occ, S, X)
        dnorm = float(np.sqrt(0.5 * (np.mean(ga * ga) + np.mean(gb * gb))))
        dE = E - E_old
        log.append({"iter": it, "energy": float(E), "dE": float(dE), "dnorm": dnorm})
        if verbose:
            print(f"  @UHF iter {it:3d}: {E:20.14f} {dE: .3e} {dnorm: .3e}")
        if abs(dE) < e_conv and dnorm < d_conv:
            converged = True
            break
        E_old = E
        F2 = np.stack((Fa, Fb))
        if it >= diis_start:
            diis.add(F2, np.stack((ga, gb)))
            F2 = diis.extrapolate() if len(diis.F) >= 2 else F2
        Ca = X @ np.linalg.eigh(X.T @ F2[0] @ X)[1]
        Cb = X @ np.linalg.eigh(X.T @ F2[1] @ X)[1]
    res = UHFResult(energies[-1], energies, it, converged, Ca, Cb, Da, Db, nalpha, nbeta,
                    {"total_s": time.perf_counter() - t0, "jk_s": t_jk}, log)
    if not converged and fail_on_maxiter:
        raise SCFConvergenceError(f"Could not converge UHF iterations in {maxiter} iterations.", res)
    return res
