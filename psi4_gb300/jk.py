"""psi4.core.JK-shaped front end of the GB300 DF-JK engine.

``GpuDFJK`` mirrors the JK API psi4's SCF drives (psi4/src/export_fock.cc:49-97,
psi4/src/psi4/libfock/jk.h:232-589): ``initialize()``, ``C_left_add`` / ``C_right_add`` /
``C_add`` / ``C_clear``, ``compute()``, ``J()``, ``K()``, ``D()``, ``memory_estimate()``,
``print_header()``, ``set_do_J`` / ``set_do_K`` / ``set_cutoff`` / ``set_memory``.  Like
``MemDFJK`` (psi4/src/psi4/libfock/MemDFJK.cc) it builds B = J^-1/2 (P|mn) once in
``initialize()`` (``preiterations``) and then serves every ``compute()`` from HBM.

Only lr-symmetric and non-symmetric C pairs (``C_right_add``) are served, as MemDFJK does;
every compute goes through libgdfjk.so — there is no CPU path.  Errors raise
``GdfjkError`` (a ``RuntimeError``, as psi4's PSIEXCEPTION surfaces in Python).

Extra knobs of this engine: ``set_precision("fp64" | "fp64-emulated" | "mixed")`` and
``set_incremental(True)`` (mixed form: K += K(dD) over the previous build).  "fp64-emulated"
computes K to FP64 accuracy from BF16 tensor-core products of 7-bit digit slices.
"""
from __future__ import annotations

import ctypes
import time

import numpy as np

from . import _jkabi as abi
from . import _native
from .dfhelper import DEFAULT_CONDITION, DEFAULT_CUTOFF, DFTensor, build_df_tensor


class GdfjkError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"gdfjk error {code}: {msg}")
        self.code = code


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


class DFJKEngine:
    """Owner of one ``gdfjk_t`` handle (one device, one stream; B resident in HBM, or with
    ``flags=abi.B_HOST`` in pinned Grace memory that the kernels read over NVLink-C2C)."""

    def __init__(self, nbf: int, naux: int, pair_mask: np.ndarray | None = None, device: int = 0, flags: int = 0):
        self.L = _native.jk_lib()
        self.nbf, self.naux = int(nbf), int(naux)
        self.device = int(device)
        h = ctypes.c_void_p()
        self._mask = None
        if pair_mask is not None:
            self._mask = np.ascontiguousarray(pair_mask, dtype=np.uint8)
            assert self._mask.shape == (nbf, nbf)
        rc = self.L.gdfjk_create(device, self.nbf, self.naux, _p(self._mask), flags, ctypes.byref(h))
        if rc != 0:
            raise GdfjkError(rc, self.L.gdfjk_last_error(None).decode())
        self.h = h

    def _check(self, rc):
        if rc != 0:
            raise GdfjkError(rc, self.L.gdfjk_last_error(self.h).decode())

    # ---- B upload
    def upload_qtri(self, B_tri: np.ndarray):
        B = np.ascontiguousarray(B_tri, dtype=np.float64)
        assert B.shape == (self.naux, self.nbf * (self.nbf + 1) // 2)
        self._check(self.L.gdfjk_upload_B(self.h, _p(B), abi.LAYOUT_QTRI, None, None, None))

    def upload_pqq(self, Ppq: np.ndarray, sparsity):
        Ppq = np.ascontiguousarray(Ppq, dtype=np.float64)
        bs = np.ascontiguousarray(sparsity.big_skips, dtype=np.int64)
        ss = np.ascontiguousarray(sparsity.small_skips, dtype=np.int64)
        fi = np.ascontiguousarray(sparsity.fun_index, dtype=np.int64)
        self._check(self.L.gdfjk_upload_B(self.h, _p(Ppq), abi.LAYOUT_PQQ, _p(bs), _p(ss), _p(fi)))

    def upload_device(self, ptr: int):
        """B already in device memory as the Q-major packed triangle (e.g. a torch tensor)."""
        self._check(self.L.gdfjk_upload_B_device(self.h, ctypes.c_void_p(ptr)))

    def upload_block(self, rows: np.ndarray, q0: int):
        """Rows q0 .. q0+len(rows)-1 of the Q-major packed triangle from host memory; blocks in
        order from q0 = 0, ready once the last row has been uploaded."""
        rows = np.ascontiguousarray(rows, dtype=np.float64)
        self._check(self.L.gdfjk_upload_B_block(self.h, _p(rows), int(q0), int(rows.shape[0])))

    def trim(self):
        """Release the tensor-core forms' derived copies of B (rebuilt on next use)."""
        self._check(self.L.gdfjk_trim(self.h))

    def metric_contract(self, metric_ptr: int, pmn_ptr: int, ncols: int, out_ptr: int, ldp: int | None = None,
                        ldb: int | None = None, accumulate: bool = False):
        """B (+)= metric (P|mn) on the tensor cores to FP64 accuracy, all device pointers:
        metric naux x naux, (P|mn) naux x ncols (leading dimension ldp), B naux x ncols (ldb);
        DFHelper::contract_metric_AO_core_symm's product (dfhelper.cc:1653-1678).  With the
        packed-triangle column order, B is ready for `upload_device`."""
        ldp = ncols if ldp is None else ldp
        ldb = ncols if ldb is None else ldb
        self._check(self.L.gdfjk_metric_contract_device(self.h, ctypes.c_void_p(metric_ptr), ctypes.c_void_p(pmn_ptr),
                                                        int(ncols), int(ldp), ctypes.c_void_p(out_ptr), int(ldb),
                                                        1 if accumulate else 0))

    def gemm(self, A_ptr: int, lda: int, B_ptr: int, ldb: int, C_ptr: int, ldc: int, M: int, N: int, K: int,
             transb: bool = False, accumulate: bool = False):
        """C (+)= A op(B) on the tensor cores to FP64 accuracy (device pointers, row-major;
        op(B) = B^T with transb, B then N x K)."""
        self._check(self.L.gdfjk_gemm_device(self.h, 1 if transb else 0, int(M), int(N), int(K), ctypes.c_void_p(A_ptr),
                                             int(lda), ctypes.c_void_p(B_ptr), int(ldb), ctypes.c_void_p(C_ptr), int(ldc),
                                             1 if accumulate else 0))

    def upload_device_block(self, ptr: int, q0: int, nq: int):
        """Rows q0 .. q0+nq-1 of the packed triangle already in device memory."""
        self._check(self.L.gdfjk_upload_B_device_block(self.h, ctypes.c_void_p(ptr), int(q0), int(nq)))

    # ---- builds
    def compute(self, C_left, C_right=None, mode=abi.DO_J | abi.DO_K, want_D=False):
        Cl = np.ascontiguousarray(C_left, dtype=np.float64)
        if Cl.ndim != 2 or Cl.shape[0] != self.nbf:
            raise GdfjkError(abi.GDFJK_ERR_ARG, f"C_left must be nbf x nocc with nbf={self.nbf}")
        Cr = None
        if C_right is not None:
            Cr = np.ascontiguousarray(C_right, dtype=np.float64)
            if Cr.shape != Cl.shape:
                raise GdfjkError(abi.GDFJK_ERR_ARG, "JK: C_left/C_right MO zip index size mismatch!")
        nocc = Cl.shape[1]
        J = np.empty((self.nbf, self.nbf))
        K = np.empty((self.nbf, self.nbf))
        D = np.empty((self.nbf, self.nbf)) if want_D else None
        self._check(self.L.gdfjk_compute(self.h, _p(Cl) if nocc else None, _p(Cr) if (Cr is not None and nocc) else None,
                                         nocc, max(nocc, 1), mode, _p(D), _p(J), _p(K)))
        return J, K, D

    def compute_wK(self, right: "DFJKEngine", C_left, C_right=None, mode=0):
        """wK = sum_Q (L_Q C_left)(R_Q C_right)^T with L = this engine's tensor (J^-1 (Q|mn)) and
        R = `right`'s ((Q|w|mn)); C_right None: lr-symmetric, symmetrised like MemDFJK.
        mode: 0 (native FP64) or abi.EMULATED."""
        Cl = np.ascontiguousarray(C_left, dtype=np.float64)
        Cr = None if C_right is None else np.ascontiguousarray(C_right, dtype=np.float64)
        nocc = Cl.shape[1]
        wK = np.empty((self.nbf, self.nbf))
        self._check(self.L.gdfjk_compute_wK(self.h, right.h, _p(Cl) if nocc else None,
                                            _p(Cr) if (Cr is not None and nocc) else None, nocc, max(nocc, 1),
                                            int(mode), _p(wK)))
        return wK

    def compute_incremental(self, C, U, npos, mode=abi.DO_J | abi.DO_K | abi.MIXED, reset=False):
        """Precision form: J (FP64) from C; K = K_prev + sum_Q B_Q (U+U+^T - U-U-^T) B_Q in
        split BF16 with FP32 accumulation (K_prev = 0 when reset).  Without MIXED in mode,
        K is a full FP64 build from C that becomes the base of later increments."""
        C = np.ascontiguousarray(C, dtype=np.float64)
        U = np.ascontiguousarray(U, dtype=np.float64)
        nocc, nu = C.shape[1], U.shape[1]
        J = np.empty((self.nbf, self.nbf))
        K = np.empty((self.nbf, self.nbf))
        m = mode | (abi.RESET if reset else 0)
        self._check(self.L.gdfjk_compute_incremental(self.h, _p(C) if nocc else None, nocc, max(nocc, 1),
                                                     _p(U) if nu else None, nu, int(npos), max(nu, 1), m, _p(J), _p(K)))
        return J, K

    def compute_incremental_device(self, C_ptr, nocc, ldc, U_ptr, nu, npos, ldu, mode, J_ptr, K_ptr):
        """gdfjk_compute_incremental_device: device buffers, asynchronous on the engine's stream."""
        vp = lambda x: None if x is None else ctypes.c_void_p(int(x))
        self._check(self.L.gdfjk_compute_incremental_device(self.h, vp(C_ptr), int(nocc), int(ldc), vp(U_ptr), int(nu),
                                                            int(npos), int(ldu), int(mode), vp(J_ptr), vp(K_ptr)))

    def compute_device(self, Cl_ptr, Cr_ptr, nocc, ldc, mode, D_ptr, J_ptr, K_ptr):
        vp = lambda x: None if x is None else ctypes.c_void_p(int(x))
        self._check(self.L.gdfjk_compute_device(self.h, vp(Cl_ptr), vp(Cr_ptr), int(nocc), int(ldc), int(mode), vp(D_ptr),
                                                vp(J_ptr), vp(K_ptr)))

    def backward(self, C, gJ, gK, want_dC=True, want_gamma=True):
        C = np.ascontiguousarray(C, dtype=np.float64)
        nocc = C.shape[1]
        gJ = np.ascontiguousarray(gJ, dtype=np.float64)
        gK = np.ascontiguousarray(gK, dtype=np.float64)
        dC = np.empty_like(C) if want_dC else None
        G = np.empty((self.naux, self.nbf * (self.nbf + 1) // 2)) if want_gamma else None
        self._check(self.L.gdfjk_backward(self.h, _p(C), nocc, max(nocc, 1), _p(gJ), _p(gK), _p(dC), _p(G), 0))
        return dC, G

    def backward_gamma_device(self, C_ptr, nocc, ldc, gJ_ptr, gK_ptr, G_ptr, ldg, col_map_ptr=None, batch_q=0):
        """gdfjk_backward_gamma_device: Gamma = dE/dB alone over aux batches, into a device
        array (packed-triangle columns or col_map's), device C / gJ / gK."""
        vp = lambda x: None if x is None else ctypes.c_void_p(int(x))
        self._check(self.L.gdfjk_backward_gamma_device(self.h, vp(C_ptr), int(nocc), int(ldc), vp(gJ_ptr), vp(gK_ptr),
                                                       vp(col_map_ptr), int(ldg), vp(G_ptr), int(batch_q)))

    def backward_device(self, C_ptr, nocc, ldc, gJ_ptr, gK_ptr, dC_ptr, G_ptr):
        vp = lambda x: None if x is None else ctypes.c_void_p(int(x))
        self._check(self.L.gdfjk_backward(self.h, vp(C_ptr), int(nocc), int(ldc), vp(gJ_ptr), vp(gK_ptr), vp(dC_ptr),
                                          vp(G_ptr), 1))

    def synchronize(self, timeout_s=600.0):
        self._check(self.L.gdfjk_synchronize(self.h, float(timeout_s)))

    def stream(self) -> int:
        return int(self.L.gdfjk_stream(self.h) or 0)

    def timings(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        self._check(self.L.gdfjk_last_timings(self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"j_ms": a.value, "k_transform_ms": b.value, "k_contract_ms": c.value}

    @staticmethod
    def query_memory(nbf, naux, max_nocc, flags=0) -> int:
        L = _native.jk_lib()
        out = ctypes.c_size_t()
        rc = L.gdfjk_query_memory(int(nbf), int(naux), int(max_nocc), int(flags), ctypes.byref(out))
        if rc != 0:
            raise GdfjkError(rc, L.gdfjk_last_error(None).decode())
        return out.value

    def close(self):
        if getattr(self, "h", None):
            self.L.gdfjk_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_POOL = None


def _host_pool():
    """One worker thread for host work that overlaps a GPU call (numpy's LAPACK and the
    engine's ctypes calls both release the interpreter lock)."""
    global _POOL
    if _POOL is None:
        from concurrent.futures import ThreadPoolExecutor

        _POOL = ThreadPoolExecutor(max_workers=1, thread_name_prefix="gdfjk-host")
    return _POOL


def _timed_factor(C_new, C_old):
    t = time.perf_counter()
    U, npos = density_difference_factor(C_new, C_old)
    return U, npos, time.perf_counter() - t


def density_difference_factor(C_new, C_old, tol=1e-13):
    """Signed low-rank factor of dD = C_new C_new^T - C_old C_old^T.

    QR of [C_new, C_old] = Q R gives dD = Q (R S R^T) Q^T with S = diag(+1.., -1..); the small
    symmetric R S R^T = W diag(lam) W^T then gives dD = U+ U+^T - U- U-^T with
    U = Q W |lam|^1/2, positive eigenvalues first: orthogonal columns of norm |lam|^1/2, so the
    split-precision increment's rounding scales with dD itself (a triangular LDL^T factor of
    R S R^T was tried: cheaper, but its non-orthogonal columns cancel, and at C100H202 the SCF
    then needed two more FP64 builds).  Eigenvalues below `tol` are dropped.
    Returns (U, npos)."""
    A = np.hstack([C_new, C_old])
    Q, R = np.linalg.qr(A)
    sgn = np.concatenate([np.ones(C_new.shape[1]), -np.ones(C_old.shape[1])])
    lam, W = np.linalg.eigh((R * sgn) @ R.T)
    keep = np.abs(lam) > tol
    lam, W = lam[keep], W[:, keep]
    order = np.argsort(-lam)
    lam, W = lam[order], W[:, order]
    U = (Q @ W) * np.sqrt(np.abs(lam))
    return np.ascontiguousarray(U), int((lam > 0).sum())


def build_jk(primary, aux, molecule, options: dict | None = None, device: int = 0) -> "GpuDFJK":
    """JK::build_JK for SCF_TYPE MEM_DF (psi4/src/psi4/libfock/jk.cc:72-160) with the options
    that reach MemDFJK, applied as psi4 applies them:
      SCREENING       CSAM (default), SCHWARZ or NONE: the Schwarz cutoff is INTS_TOLERANCE, or
                      0 for NONE (jk.cc:112); DENSITY raises psi4's error unless DF_SCF_GUESS
                      (jk.cc:83-109) — MemDFJK itself has no density screening
      INTS_TOLERANCE  default 1e-12;  DF_FITTING_CONDITION  default 1e-10
      SCF_SUBTYPE     AUTO, INCORE or OUT_OF_CORE: psi4's MemDFJK does not read it; here
                      OUT_OF_CORE keeps B in Grace memory (GDFJK_B_HOST), with the same results."""
    o = {"SCREENING": "CSAM", "INTS_TOLERANCE": DEFAULT_CUTOFF, "DF_SCF_GUESS": True, "SCF_SUBTYPE": "AUTO",
         "DF_FITTING_CONDITION": DEFAULT_CONDITION}
    o.update({str(k).upper(): v for k, v in (options or {}).items()})
    screening = str(o["SCREENING"]).upper()
    if screening not in ("SCHWARZ", "CSAM", "DENSITY", "NONE"):
        raise ValueError(f"SCREENING must be SCHWARZ, CSAM, DENSITY or NONE, not {screening}")
    if screening == "DENSITY" and not o["DF_SCF_GUESS"]:
        raise RuntimeError("SCREENING=DENSITY has not been implemented for MEM_DF.")
    subtype = str(o["SCF_SUBTYPE"]).upper()
    if subtype not in ("AUTO", "INCORE", "OUT_OF_CORE"):
        raise ValueError("Invalid SCF_SUBTYPE option! The choices for SCF_SUBTYPE are AUTO, INCORE, and OUT_OF_CORE.")
    jk = GpuDFJK(primary, aux, molecule, device=device)
    jk.set_cutoff(0.0 if screening == "NONE" else float(o["INTS_TOLERANCE"]))
    jk.set_condition(float(o["DF_FITTING_CONDITION"]))
    jk.set_b_host(subtype == "OUT_OF_CORE")
    return jk


class GpuDFJK:
    """A drop-in for psi4's MemDFJK in an RHF loop, served by the GB300 engine."""

    def __init__(self, primary=None, aux=None, molecule=None, df_tensor: DFTensor | None = None, device: int = 0):
        self.primary, self.aux, self.molecule = primary, aux, molecule
        self.df = df_tensor
        self.device = device
        self.cutoff = DEFAULT_CUTOFF
        self.condition = DEFAULT_CONDITION
        self.memory = 32_000_000  # doubles, psi4's JK default (256 MB)
        self.do_J = True
        self.do_K = True
        self.precision = "fp64"
        self.incremental = False
        self.print_level = 1
        self.engine: DFJKEngine | None = None
        self.b_host = False  # B in pinned Grace memory (GDFJK_B_HOST)
        self.do_wK = False
        self.omega = 0.0
        self.wk_engines: tuple[DFJKEngine, DFJKEngine] | None = None
        self._wK = []
        self._Cl, self._Cr = [], []
        self._J, self._K, self._D = [], [], []
        self.last_timings = {}
        self._C_prev = None
        self.last_rank = 0

    # psi4: core.JK.build(orbital_basis, aux, jk_type=...)
    @staticmethod
    def build(primary, aux, molecule, **kw) -> "GpuDFJK":
        return GpuDFJK(primary, aux, molecule, **kw)

    @staticmethod
    def from_tensor(df: DFTensor, device: int = 0) -> "GpuDFJK":
        return GpuDFJK(df_tensor=df, device=device)

    @staticmethod
    def from_engine(engine: "DFJKEngine") -> "GpuDFJK":
        """A JK object over an engine whose B is already uploaded (e.g. B built on the device
        in blocks); initialize() is then a no-op."""
        jk = GpuDFJK(device=engine.device)
        jk.engine = engine
        return jk

    def name(self):
        return "GpuDFJK"

    def set_do_J(self, v):
        self.do_J = bool(v)

    def set_do_K(self, v):
        self.do_K = bool(v)

    def set_cutoff(self, c):
        self.cutoff = float(c)

    def set_condition(self, c):
        self.condition = float(c)

    def set_memory(self, doubles):
        self.memory = int(doubles)

    def set_print(self, p):
        self.print_level = int(p)

    def set_do_wK(self, v: bool):
        """Also build the long-range exchange wK (MemDFJK with do_wK, DFHelper::compute_wK)."""
        self.do_wK = bool(v)

    def set_omega(self, w: float):
        self.omega = float(w)

    def wK(self):
        return self._wK

    def set_b_host(self, v: bool):
        """Keep B in pinned host (Grace) memory, read over NVLink-C2C: results are unchanged,
        HBM holds only the workspaces (and the tensor-core forms' derived copies)."""
        self.b_host = bool(v)

    def set_precision(self, p: str):
        if p not in ("fp64", "fp64-emulated", "mixed"):
            raise ValueError("precision must be 'fp64', 'fp64-emulated' or 'mixed'")
        self.precision = p

    def set_incremental(self, v: bool):
        self.incremental = bool(v)

    def reset_incremental(self):
        """Forget the previous density: the next mixed build is a full build."""
        self._C_prev = None

    def C1(self):
        return True

    def memory_estimate(self) -> int:
        """Device bytes / 8, in doubles like psi4's JK::memory_estimate (jk.h:398)."""
        nbf = self.df.nbf if self.df is not None else self.primary.nbf
        naux = self.df.naux if self.df is not None else self.aux.nbf
        flags = {"mixed": abi.MIXED, "fp64-emulated": abi.EMULATED}.get(self.precision, 0)
        flags |= abi.B_HOST if self.b_host else 0
        total = DFJKEngine.query_memory(nbf, naux, nbf, flags)
        if self.do_wK:  # two more tensors (J^-1 (Q|mn), (Q|w|mn)), each in its own engine
            total += 2 * (total - DFJKEngine.query_memory(nbf, naux, nbf, flags | abi.B_HOST))
        return total // 8

    def initialize(self):
        """preiterations(): build B on the host, upload it to HBM once."""
        if self.engine is not None and self.df is None:
            return
        if self.df is None:
            self.df = build_df_tensor(self.molecule, self.primary, self.aux, self.cutoff, self.condition)
        df = self.df
        self.engine = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask, device=self.device,
                                 flags=abi.B_HOST if self.b_host else 0)
        self.engine.upload_pqq(df.to_pQq(), df.sparsity)
        if self.do_wK:
            # prepare_AO_wK_core: J^-1 (Q|mn) and (Q|w|mn), one engine each
            if self.molecule is None or not self.omega > 0:
                raise GdfjkError(abi.GDFJK_ERR_STATE, "JK: wK needs the molecule and omega > 0")
            from .dfhelper import build_wk_tensors
            from .ints import Integrals

            m1, w = build_wk_tensors(df, Integrals(self.molecule, self.primary, self.aux), self.omega, self.condition)
            engines = []
            for t in (m1, w):
                e = DFJKEngine(df.nbf, df.naux, df.sparsity.pair_mask, device=self.device,
                               flags=abi.B_HOST if self.b_host else 0)
                e.upload_qtri(t.B_tri)
                engines.append(e)
            self.wk_engines = (engines[0], engines[1])

    def print_header(self):
        if self.print_level:
            sp = self.df.sparsity if self.df is not None else None
            print("  ==> GpuDFJK: Density-Fitted J/K Matrices (GB300) <==\n")
            print(f"    J tasked:           {'Yes' if self.do_J else 'No':>11s}")
            print(f"    K tasked:           {'Yes' if self.do_K else 'No':>11s}")
            print(f"    Precision:          {self.precision:>11s}")
            print(f"    Schwarz Cutoff:     {self.cutoff:11.0E}")
            if sp is not None:
                print(f"    Mask sparsity (%):  {100.0 * sp.sparsity:11.4f}")
            print(f"    Fitting Condition:  {self.condition:11.0E}\n")

    def C_clear(self):
        self._Cl, self._Cr = [], []

    def C_left_add(self, C):
        self._Cl.append(np.asarray(C, dtype=np.float64))

    def C_right_add(self, C):
        self._Cr.append(np.asarray(C, dtype=np.float64))

    def C_add(self, C):
        self.C_left_add(C)
        self.C_right_add(C)

    def compute(self):
        if self.engine is None:
            raise GdfjkError(abi.GDFJK_ERR_STATE, "JK: compute() before initialize()")
        lr_symmetric = len(self._Cl) > 0 and len(self._Cr) == 0
        if not lr_symmetric and len(self._Cr) != len(self._Cl):
            raise GdfjkError(abi.GDFJK_ERR_ARG, "JK: C_left/C_right count mismatch")
        mode = (abi.DO_J if self.do_J else 0) | (abi.DO_K if self.do_K else 0)
        if self.precision == "mixed" and lr_symmetric:
            mode |= abi.MIXED
            if self.incremental:
                mode |= abi.INCREMENTAL
        # the emulated form serves densities with up to 1024 occupied columns (lr-symmetric or
        # C_left != C_right); wider ones take the native FP64 K
        emu = abi.EMULATED if (self.precision == "fp64-emulated" and
                               all(C.shape[1] <= 1024 for C in self._Cl)) else 0
        mode |= emu
        self._J, self._K, self._D = [], [], []
        self._wK = []
        if self.do_wK and self.wk_engines is not None:
            # DFHelper::compute_wK for every density (native FP64, or the emulated form with it)
            left, right = self.wk_engines
            for i, Cl in enumerate(self._Cl):
                Cr = None if lr_symmetric else self._Cr[i]
                self._wK.append(left.compute_wK(right, Cl, Cr, mode=emu))
        single = lr_symmetric and len(self._Cl) == 1 and self._Cl[0].shape[1] > 0
        if self.precision in ("fp64", "fp64-emulated") and self.incremental and single and self.do_K:
            # FP64 re-anchor of the precision form: full FP64 K, kept as the incremental base
            C = self._Cl[0]
            J, K = self.engine.compute_incremental(C, C, C.shape[1],
                                                   mode=(abi.DO_J if self.do_J else 0) | abi.DO_K | emu)
            self._C_prev = C.copy()
            self._J.append(J if self.do_J else None)
            self._K.append(K)
            self._D = None
            self.last_timings = self.engine.timings()
            return
        if self.precision == "mixed" and single and self.do_K:
            # the precision form: K from the split-BF16 tensor-core path, incremental over dD.
            # The FP64 J of the new orbitals runs on the GPU while the host factors dD (both
            # calls release the interpreter lock), then the K increment.
            C = self._Cl[0]
            if self.incremental and self._C_prev is not None and self._C_prev.shape == C.shape:
                t0 = time.perf_counter()
                fut = _host_pool().submit(_timed_factor, C, self._C_prev)
                J = self.engine.compute(C, mode=abi.DO_J)[0] if self.do_J else None
                t1 = time.perf_counter()
                U, npos, t_factor = fut.result()
                t2 = time.perf_counter()
                _, K = self.engine.compute_incremental(C, U, npos, mode=abi.DO_K | abi.MIXED, reset=False)
                t3 = time.perf_counter()
                self.last_rank = U.shape[1]
                self.last_increment_s = {"j": t1 - t0, "factor_host": t_factor, "wait_for_factor": t2 - t1,
                                         "k_increment": t3 - t2}
            else:
                J, K = self.engine.compute_incremental(C, C, C.shape[1], mode=(abi.DO_J if self.do_J else 0) | abi.DO_K
                                                       | abi.MIXED, reset=True)
                J = J if self.do_J else None
                self.last_rank = C.shape[1]
            self._C_prev = C.copy()
            self._J.append(J)
            self._K.append(K)
            self._D = None
            self.last_timings = self.engine.timings()
            return
        if single:
            self._C_prev = None
            J, K, _ = self.engine.compute(self._Cl[0], None, mode=mode)
            self._J.append(J if self.do_J else None)
            self._K.append(K if self.do_K else None)
            self._D = None
            self.last_timings = self.engine.timings()
            return
        self._C_prev = None
        for i, Cl in enumerate(self._Cl):
            Cr = None if lr_symmetric else self._Cr[i]
            if Cr is not None and Cr.shape[1] != Cl.shape[1]:
                raise GdfjkError(abi.GDFJK_ERR_ARG, "JK: C_left/C_right MO zip index size mismatch!")
            J, K, D = self.engine.compute(Cl, Cr, mode=mode, want_D=True)
            self._J.append(J if self.do_J else None)
            self._K.append(K if self.do_K else None)
            self._D.append(D)
        self.last_timings = self.engine.timings()

    def J(self):
        return self._J

    def K(self):
        return self._K

    def D(self):
        if self._D is None:  # formed on request (JK::compute_D, jk.cc:314-354)
            self._D = [C @ C.T for C in self._Cl]
        return self._D

    def finalize(self):
        if self.engine is not None:
            self.engine.close()
            self.engine = None
        if self.wk_engines is not None:
            for e in self.wk_engines:
                e.close()
            self.wk_engines = None
