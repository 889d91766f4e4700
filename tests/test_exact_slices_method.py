"""The arithmetic behind the exact-slice tensor-core products, restated in
numpy (the CUDA kernels, k_tcx.cu, are checked against FP64 products on the
GPU by test_gpu_exact.py): every operand row scaled by 2^-e (e = 1 + its
largest binary exponent) and written as six balanced base-128 digits
  x = 2^e sum_s d_s 2^-7(s+1),  |d_0| <= 128, |d_s| <= 64 (s >= 1),
each exact in bf16; the 21 digit products with s + u <= 5 summed into six
accumulators J_q (q = s + u) stay integers below 2^24 in magnitude -- exact
in f32 -- for K <= 512 even when every digit takes its largest value; the
int64 combination sum_q J_q 2^(7(5-q)) times 2^(e_r + f_c - 49) then gives
(A B^T)_rc to within 2^-41 (sum_k |a_rk| max_k |b_ck| + max_k |a_rk| sum_k
|b_ck|), the truncation of the two operands' digits, plus FP64 rounding
(checked against exact rational arithmetic on small cases and long-double
products on larger ones)."""
from fractions import Fraction

import numpy as np

NS = 6
C = 64 * sum(1 << (7 * i) for i in range(5))  # offset that balances the five lower digits


def row_exponents(X):
    """1 + the largest unbiased binary exponent of each row (rows of zeros
    get 0; their digits are all zero)."""
    a = np.abs(X).max(axis=1)
    e = np.zeros(len(a), dtype=np.int64)
    nz = a > 0
    e[nz] = np.frexp(a[nz])[1]  # frexp: a = m 2^E, m in [0.5, 1): E = unbiased exponent + 1
    return e


def digits6(X, e):
    """The six digits of every element of X (rows scaled by 2^-e)."""
    # M = round(|x| 2^(42 - e)), an integer below 2^42
    M = np.rint(np.ldexp(np.abs(X), (42 - e)[:, None])).astype(np.int64)
    Mp = M + C
    sg = np.where(X < 0, -1, 1)
    d = np.empty(X.shape + (NS,), dtype=np.int64)
    d[..., 0] = sg * (Mp >> 35)
    for s in range(1, NS):
        d[..., s] = sg * (((Mp >> (7 * (5 - s))) & 127) - 64)
    return d


def exact_product(A, B):
    ea, eb = row_exponents(A), row_exponents(B)
    Ad, Bd = digits6(A, ea), digits6(B, eb)
    K = A.shape[1]
    acc = np.zeros((A.shape[0], B.shape[0]), dtype=np.int64)
    out = np.zeros(acc.shape)
    for k0 in range(0, K, 512):
        J = np.zeros((NS,) + acc.shape, dtype=np.int64)
        for q in range(NS):
            for s in range(q + 1):
                J[q] += Ad[:, k0:k0 + 512, s] @ Bd[:, k0:k0 + 512, q - s].T
        assert np.abs(J).max() < 2 ** 24  # exact in f32
        blk = sum(J[q] * (1 << (7 * (5 - q))) for q in range(NS))
        out += np.ldexp(blk.astype(np.float64), (ea[:, None] + eb[None, :] - 49))
    return out


def test_digits_reconstruct_and_fit_bf16():
    rng = np.random.default_rng(1)
    X = rng.standard_normal((64, 40)) * np.exp(rng.uniform(-30, 30, (64, 1))) * np.exp(rng.uniform(-8, 0, (64, 40)))
    e = row_exponents(X)
    d = digits6(X, e)
    assert np.abs(d[..., 0]).max() <= 128
    # balanced digits of |x| lie in [-64, 63]; the sign of x flips them
    assert np.abs(d[..., 1:]).max() <= 64
    # every digit is a small integer, exact in bf16 (8 significant bits)
    assert np.all(np.abs(d) <= 256)
    back = sum(np.ldexp(d[..., s].astype(np.float64), (e - 7 * (s + 1))[:, None]) for s in range(NS))
    rowmax = np.abs(X).max(axis=1, keepdims=True)
    assert np.all(np.abs(back - X) <= np.ldexp(rowmax, -42))


def test_worst_case_accumulators_fit_f32():
    """Every digit at its largest magnitude over K = 512: the biggest
    accumulator, J_5 (two products with a leading digit of 128 and four of
    64 x 64 per K element), stays below 2^24."""
    K = 512
    worst = [128] + [64] * 5
    for q in range(NS):
        bound = K * sum(worst[s] * worst[q - s] for s in range(q + 1))
        assert bound <= 2 ** 24, (q, bound)


def test_product_against_exact_rationals():
    rng = np.random.default_rng(2)
    A = rng.standard_normal((6, 37)) * np.exp(rng.uniform(-10, 10, (6, 1)))
    B = rng.standard_normal((5, 37)) * np.exp(rng.uniform(-10, 10, (5, 1)))
    A[2] = 0.0
    got = exact_product(A, B)
    for r in range(A.shape[0]):
        for c in range(B.shape[0]):
            ref = sum(Fraction(a) * Fraction(b) for a, b in zip(A[r], B[c]))
            bound = sum(abs(Fraction(a)) for a in A[r]) * max(abs(Fraction(b)) for b in B[c]) + \
                max(abs(Fraction(a)) for a in A[r]) * sum(abs(Fraction(b)) for b in B[c])
            assert abs(Fraction(got[r, c]) - ref) <= bound * Fraction(1, 2 ** 41) + abs(ref) * Fraction(1, 2 ** 52)


def test_product_long_k_and_wide_range():
    rng = np.random.default_rng(3)
    for m, n, K in ((16, 8, 600), (8, 8, 1100)):
        A = rng.standard_normal((m, K)) * np.exp(rng.uniform(-20, 5, (m, 1))) * np.exp(rng.uniform(-3, 3, (m, K)))
        B = rng.standard_normal((n, K)) * np.exp(rng.uniform(-5, 5, (n, 1)))
        ref = (A.astype(np.longdouble) @ B.T.astype(np.longdouble)).astype(np.float64)
        got = exact_product(A, B)
        scale = np.abs(A).max(1)[:, None] * np.abs(B).max(1)[None, :] * K
        assert np.max(np.abs(got - ref) / scale) <= 2.0 ** -40
