"""CPU model of the digit-split (Ozaki) arithmetic behind the emulated-FP64 exchange.

The engine writes a row with |x| < 2^E as v = round(x 2^(47-E)) = sum_s d_s 2^(7(6-s)) with
balanced digits d_s in [-64, 63] (7 slices), forms the 28 slice products with s + t <= 6 on
BF16 tensor cores, keeps levels 0-4 in their own FP32 accumulators (exact integer sums) and
levels 5-6 in a tail accumulator, and adds the six in double-float.  The tensor cores' FP32
accumulation rounds toward zero; this model reproduces that on the tail and checks the error
bounds and the diagonal bias the kernels rely on.
"""
import numpy as np

P = 7          # digit slices
MAX_LEVEL = 6  # highest level s + t kept
EXACT = 4      # levels 0..EXACT have their own accumulator
OFF = 64 * sum(1 << (7 * s) for s in range(P))


def row_exponent(x):
    m = np.max(np.abs(x), axis=-1)
    _, e = np.frexp(m)  # m = f 2^e with f in [0.5, 1): m < 2^e
    return np.where(m > 0, e, -100000)


def digits(x, E, p=P):
    """Balanced 7-bit digits (most significant first, p of them) of rows of x with |x| < 2^E."""
    off = 64 * sum(1 << (7 * s) for s in range(p))
    v = np.rint(np.ldexp(x, (7 * p - 2 - E)[..., None])).astype(np.int64)
    u = v + off
    assert (u >= 0).all() and (u < (1 << (7 * p))).all()
    return np.stack([((u >> (7 * (p - 1 - s))) & 127) - 64 for s in range(p)], axis=0).astype(np.float64)


def _f32_rz(x):
    """float64 -> float32 rounding toward zero (the tensor cores' accumulation)."""
    r = x.astype(np.float32)
    over = np.abs(r.astype(np.float64)) > np.abs(x)
    return np.where(over, np.nextafter(r, np.float32(0)), r)


def emulated_product(A, B, exact=EXACT, kstep=16, p=P, max_level=MAX_LEVEL):
    """A (m x k) @ B (n x k)^T as the kernels form it: per-row exponents of both operands,
    p digits, exact levels 0..exact, the remaining levels <= max_level in a round-toward-zero
    FP32 tail updated once per pair and 16-deep k step."""
    EA, EB = row_exponent(A), row_exponent(B)
    dA, dB = digits(A, EA, p), digits(B, EB, p)
    total = np.zeros((A.shape[0], B.shape[0]))
    for s in range(p):
        for t in range(p):
            if s + t <= exact:
                total += (dA[s] @ dB[t].T) * 2.0 ** (-7 * (s + t))  # exact integers
    tail = np.zeros_like(total, dtype=np.float32)
    pairs = [(s, t) for s in range(p) for t in range(p) if exact < s + t <= max_level]
    for k0 in range(0, A.shape[1], kstep):
        for s, t in pairs:
            term = (dA[s][:, k0:k0 + kstep] @ dB[t][:, k0:k0 + kstep].T) * 2.0 ** (-7 * (s + t))
            tail = _f32_rz(tail.astype(np.float64) + term)
    return np.ldexp(total + tail, EA[:, None] + EB[None, :] - 10)


def test_digit_reconstruction():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((50, 300)) * np.exp(rng.uniform(-20, 5, size=(50, 1)))
    E = row_exponent(x)
    d = digits(x, E)
    assert d.min() >= -64 and d.max() <= 63
    v = sum(d[s] * 2.0 ** (7 * (P - 1 - s)) for s in range(P))
    back = np.ldexp(v, (E - 47)[:, None])
    assert (np.abs(back - x).max(axis=1) <= np.ldexp(1.0, E - 48)).all()


def test_emulated_product_accuracy():
    rng = np.random.default_rng(2)
    for k in (64, 1024):
        A = rng.standard_normal((24, k)) * rng.uniform(0.01, 1, size=(24, 1))
        B = rng.standard_normal((16, k))
        err = np.abs(emulated_product(A, B) - A @ B.T)
        scale = np.abs(A).max(axis=1)[:, None] * np.abs(B).max(axis=1)[None, :] * np.sqrt(k)
        assert (err / scale).max() < 2.0**-42  # measured ~2^-44


def test_diagonal_bias_needs_level4_accumulator():
    """Sums of squares (the diagonal of K) of rows whose elements span many binades: with
    level 4 in the round-toward-zero tail the result is biased low; with its own accumulator
    the bias is gone."""
    rng = np.random.default_rng(3)
    k = 1024
    X = rng.standard_normal((8, k)) * np.exp(rng.uniform(-12, 0, size=(8, k)))
    ref = np.einsum("ik,ik->i", X, X)
    biased = np.diag(emulated_product(X, X, exact=3)) / ref - 1
    fixed = np.diag(emulated_product(X, X, exact=4)) / ref - 1
    assert biased.max() < 0  # every diagonal element low
    assert np.abs(fixed).max() < np.abs(biased).min() / 10


def test_exact_level_bounds():
    """Levels 0-3 stay below 2^24 units for any digits over a 1024-term run; level 4 (5 pairs)
    up to 819 terms in the worst case."""
    for L in range(4):
        assert (L + 1) * 1024 * 64 * 64 <= 2**24
    assert 5 * 819 * 64 * 64 <= 2**24


def test_metric_contraction_needs_eight_digits(ints_built):
    """The metric contraction B = J^-1/2 (P|mn) on real integrals (water cc-pVTZ): J^-1/2 has
    entries ~50 that cancel to |B| <= 1.06, and the digit error scales with row and column
    maxima, not with each term.  The K build's scheme (7 digits, levels <= 6, levels 0-4 exact)
    leaves ~7e-11 in B; the product kernel's (8 digits, levels <= 8, levels 0-5 exact) ~4e-14."""
    from tests.helpers import system

    mol, pb, ab, ints, df = system("h2o_scf2", "cc-pvtz")
    A = ints.three_index(shell_mask=df.sparsity.shell_mask)
    r, c = np.tril_indices(df.nbf)
    A[:, ~df.sparsity.pair_mask[r, c]] = 0.0
    assert df.naux <= 1024  # one accumulation run
    e7 = np.abs(emulated_product(df.Jmhalf, A.T.copy(), exact=4, p=7, max_level=6) - df.B_tri).max()
    e8 = np.abs(emulated_product(df.Jmhalf, A.T.copy(), exact=5, p=8, max_level=8) - df.B_tri).max()
    print(f"water cc-pVTZ metric contraction: 7 digits {e7:.2e}, 8 digits {e8:.2e}")
    assert e7 > 1e-11
    assert e8 < 1e-12

