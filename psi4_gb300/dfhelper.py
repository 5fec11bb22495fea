"""Host-side preparation of the metric-contracted 3-index tensor B = J^-1/2 (P|mn).

This is the host half of psi4's ``DFHelper::initialize`` for the in-core (STORE) JK path
(psi4/src/psi4/lib3index/dfhelper.cc:149-215).  It produces B in the two layouts the
device engine accepts through ``gdfjk_upload_B``:

* **DFHelper's pQq layout** (dfhelper.cc:1671-1673):
  ``Ppq[big_skips[m] + Q*small_skips[m] + fun_index[m, n] - 1] = B[Q, m, n]`` for every
  significant n (full square over significant pairs, p-major);
* **Q-major packed lower triangle**: ``B_tri[Q, m*(m+1)/2 + n]`` for m >= n with
  insignificant pairs held at zero.

Screening and indexing follow ``DFHelper::prepare_sparsity`` (dfhelper.cc:299-420): a pair
(m, n) is significant when max|(mn|mn)| >= cutoff^2 / max_all.  The metric power follows
``Matrix::power`` (psi4/src/psi4/libmints/matrix.cc:2370-2415): eigenvalues with
|lambda| < condition * max|lambda| are dropped for negative powers.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .basis import BasisSet
from .ints import Integrals
from .molecule import Molecule

# psi4 defaults on this path: JK cutoff 1e-12 (jk.cc:258, INTS_TOLERANCE read_options.cc:1502);
# DF_FITTING_CONDITION 1e-10 (read_options.cc:1734, applied at jk.cc:65).
DEFAULT_CUTOFF = 1.0e-12
DEFAULT_CONDITION = 1.0e-10


@dataclass
class Sparsity:
    nbf: int
    naux: int
    fun_index: np.ndarray          # (nbf, nbf) int64: running count of significant n in row m, 0 if screened
    small_skips: np.ndarray        # (nbf+1,) significant n per row m; [nbf] = total
    big_skips: np.ndarray          # (nbf+1,) row offsets in the pQq layout
    symm_small_skips: np.ndarray   # (nbf,) significant n >= m per row
    symm_ignored_columns: np.ndarray  # (nbf,) significant n < m per row
    symm_big_skips: np.ndarray     # (nbf+1,)
    shell_mask: np.ndarray         # (nshell, nshell) uint8
    pair_mask: np.ndarray          # (nbf, nbf) bool

    @property
    def s_sq(self) -> int:
        return int(self.small_skips[: self.nbf].sum())

    @property
    def s_tri(self) -> int:
        return (self.s_sq + self.nbf) // 2

    @property
    def sparsity(self) -> float:
        return 1.0 - self.s_sq / float(self.nbf * self.nbf)


def prepare_sparsity(fun_max: np.ndarray, shell_max: np.ndarray, cutoff: float, naux: int) -> Sparsity:
    nbf = fun_max.shape[0]
    max_val = float(fun_max.max()) if fun_max.size else 0.0
    tol = cutoff * cutoff / max_val if max_val > 0 else 0.0
    shell_mask = (shell_max >= tol).astype(np.uint8)
    pair = fun_max >= tol
    fun_index = np.where(pair, np.cumsum(pair, axis=1), 0).astype(np.int64)
    small = np.zeros(nbf + 1, dtype=np.int64)
    small[:nbf] = pair.sum(1)
    small[nbf] = small[:nbf].sum()
    big = np.zeros(nbf + 1, dtype=np.int64)
    big[1:] = np.cumsum(small[:nbf] * naux)
    upper = np.triu(pair)
    ssmall = upper.sum(1).astype(np.int64)
    sign = (pair & ~upper).sum(1).astype(np.int64)
    sbig = np.zeros(nbf + 1, dtype=np.int64)
    sbig[1:] = np.cumsum(ssmall * naux)
    return Sparsity(nbf, naux, fun_index, small, big, ssmall, sign, sbig, shell_mask, pair)


def dense_sparsity(nbf: int, naux: int, nshell: int = 1) -> Sparsity:
    """Every pair significant (no screening)."""
    return prepare_sparsity(np.ones((nbf, nbf)), np.ones((nshell, nshell)), 0.0, naux)


def metric_power(M: np.ndarray, power: float, condition: float) -> np.ndarray:
    """Matrix::power restated: eigendecompose, drop |lambda| < condition * max|lambda| for
    negative powers (and non-finite results), rebuild V diag(lambda^power) V^T."""
    w, V = np.linalg.eigh(M)
    max_a = max(abs(w[-1]), abs(w[0]))
    a = np.zeros_like(w)
    for i, lam in enumerate(w):
        if power < 0.0 and abs(lam) < condition * max_a:
            a[i] = 0.0
        else:
            with np.errstate(all="ignore"):
                v = lam**power if lam > 0 or float(power).is_integer() else np.nan
            a[i] = v if np.isfinite(v) else 0.0
    return (V * a) @ V.T


@dataclass
class DFTensor:
    """B = J^-1/2 (P|mn) for a molecule, with the screening tables."""

    nbf: int
    naux: int
    B_tri: np.ndarray   # (naux, nbf(nbf+1)/2), screened pairs zero
    sparsity: Sparsity
    metric: np.ndarray  # (P|Q)
    Jmhalf: np.ndarray

    def to_pQq(self) -> np.ndarray:
        """DFHelper's in-core layout (dfhelper.cc:1671-1673)."""
        sp = self.sparsity
        nbf, naux = self.nbf, self.naux
        out = np.zeros(int(sp.big_skips[nbf]))
        rows, cols = np.tril_indices(nbf)
        for m in range(nbf):
            sig = np.nonzero(sp.pair_mask[m])[0]
            if sig.size == 0:
                continue
            hi = np.maximum(sig, m)
            lo = np.minimum(sig, m)
            tri = hi * (hi + 1) // 2 + lo
            blk = self.B_tri[:, tri]  # (naux, nsig)
            out[sp.big_skips[m]: sp.big_skips[m + 1]] = blk.reshape(-1)
        return out

    def dense(self) -> np.ndarray:
        """B as (naux, nbf, nbf) — small systems only."""
        nbf = self.nbf
        full = np.zeros((self.naux, nbf, nbf))
        r, c = np.tril_indices(nbf)
        full[:, r, c] = self.B_tri
        full[:, c, r] = self.B_tri
        return full


def build_df_tensor(mol: Molecule, primary: BasisSet, aux: BasisSet, cutoff: float = DEFAULT_CUTOFF,
                    condition: float = DEFAULT_CONDITION, ints: Integrals | None = None) -> DFTensor:
    ints = ints or Integrals(mol, primary, aux)
    fun_max, shell_max = ints.schwarz()
    sp = prepare_sparsity(fun_max, shell_max, cutoff, aux.nbf)
    A = ints.three_index(shell_mask=sp.shell_mask)
    # function-level screening: screened pairs are absent from psi4's sparse tensor
    r, c = np.tril_indices(primary.nbf)
    A[:, ~sp.pair_mask[r, c]] = 0.0
    M = ints.metric()
    Jm = metric_power(M, -0.5, condition)
    B = Jm @ A
    return DFTensor(primary.nbf, aux.nbf, B, sp, M, Jm)


def build_wk_tensors(df: DFTensor, ints: Integrals, omega: float,
                     condition: float = DEFAULT_CONDITION) -> tuple[DFTensor, DFTensor]:
    """The two tensors of psi4's wK (DFHelper::prepare_AO_wK_core, dfhelper.cc:589-699, with
    MemDFJK's default wcombine = false): J^-1 (Q|mn) (metric power -1.0, dfhelper.h:357, same
    fitting condition) and the raw long-range integrals (Q|erf(w r)/r|mn), both over the
    Schwarz sparsity of `df` (screened pairs zero).  Returned as DF tensors sharing `df`'s
    tables, ready for an engine upload."""
    import dataclasses

    sp = df.sparsity
    r, c = np.tril_indices(df.nbf)
    screened = ~sp.pair_mask[r, c]
    A = ints.three_index(shell_mask=sp.shell_mask)
    A[:, screened] = 0.0
    Jinv = metric_power(df.metric, -1.0, condition)
    W = ints.three_index_erf(omega, shell_mask=sp.shell_mask)
    W[:, screened] = 0.0
    return dataclasses.replace(df, B_tri=Jinv @ A), dataclasses.replace(df, B_tri=W)

