"""The library's batched symmetric eigensolver (bgpu_diagonalise; the solver
of every density-matrix sector above 48 states) against LAPACK through
numpy.linalg.eigh, the routine family the reference calls (DSYEV,
MatrixBLAS.C:381-414).

Tolerances written here, with ||A|| the largest |eigenvalue|:
  eigenvalues within 1e-12 ||A|| of LAPACK's;
  residuals ||A v - lambda v|| within 1e-11 ||A|| for every eigenvector;
  orthogonality |V^T V - I| within 1e-12 elementwise.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def check(A, w, V):
    w0 = np.linalg.eigvalsh(A)
    na = max(np.max(np.abs(w0)), 1e-300)
    assert np.all(np.diff(w) >= 0)
    assert np.max(np.abs(w - w0)) <= 1e-12 * na, np.max(np.abs(w - w0)) / na
    res = np.linalg.norm(A @ V - V * w, axis=0)
    assert np.max(res) <= 1e-11 * na, np.max(res) / na
    n = A.shape[0]
    assert np.max(np.abs(V.T @ V - np.eye(n))) <= 1e-12


def density_like(rng, n, rank=None):
    """PSD, unit trace, eigenvalues decaying over many decades (a reduced
    density matrix); rank-deficient when rank < n."""
    r = n if rank is None else rank
    Q, _ = np.linalg.qr(rng.standard_normal((n, n)))
    lam = np.zeros(n)
    lam[:r] = np.exp(-np.linspace(0.0, 40.0, r))
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    return A / np.trace(A)


@pytest.mark.parametrize("n", [1, 2, 3, 5, 49, 64, 65, 130, 257, 700, 1000])
def test_random_symmetric(gpu_ctx, n):
    rng = np.random.default_rng(n)
    X = rng.standard_normal((n, n))
    A = 0.5 * (X + X.T)
    (w, V), = gpu_ctx.diagonalise([A])
    check(A, w, V)


@pytest.mark.parametrize("n,rank", [(97, None), (300, 60), (1000, 400)])
def test_density_like(gpu_ctx, n, rank):
    rng = np.random.default_rng(1000 + n)
    A = density_like(rng, n, rank)
    (w, V), = gpu_ctx.diagonalise([A])
    check(A, w, V)


def test_degenerate_and_diagonal(gpu_ctx):
    rng = np.random.default_rng(5)
    Q, _ = np.linalg.qr(rng.standard_normal((80, 80)))
    lam = np.repeat([0.5, 0.25, 0.0, -1.0], 20)
    A = (Q * lam) @ Q.T
    A = 0.5 * (A + A.T)
    D = np.diag(np.linspace(3.0, -2.0, 60))
    Z = np.zeros((70, 70))
    for (w, V), M in zip(gpu_ctx.diagonalise([A, D, Z]), [A, D, Z]):
        check(M, w, V)


def test_mixed_batch_is_bitwise_reproducible(gpu_ctx):
    rng = np.random.default_rng(11)
    mats = []
    for n in (50, 700, 3, 129, 64, 1):
        X = rng.standard_normal((n, n))
        mats.append(0.5 * (X + X.T))
    a = gpu_ctx.diagonalise(mats)
    b = gpu_ctx.diagonalise(mats)
    for M, (w, V), (w2, V2) in zip(mats, a, b):
        check(M, w, V)
        assert np.array_equal(w, w2) and np.array_equal(V, V2)


def test_order_limit_is_refused(gpu_ctx):
    import block_gb300

    with pytest.raises(block_gb300.BgpuError, match="order"):
        gpu_ctx.diagonalise([np.eye(4097)], vectors=False)
