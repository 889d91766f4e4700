"""Size-independent properties of sigma = H psi on the full-size config-2
superblock (synthetic 24-orbital Hamiltonian, M=500, middle bond; psi of
255 195 elements), where no oracle product is cheap enough for a test:
Hermiticity <phi|H psi> = <psi|H phi> and linearity
H(a psi + b phi) = a H psi + b H phi, to 1e-11 (relative to |phi| |H psi|
and |H(a psi + b phi)|) in FP64 and to 2e-5 in the split precision, whose
products carry a relative error of a few 1e-6; the split product matches the
FP64 one to 2e-5."""
import numpy as np
import pytest

from conftest import conf

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def big(gpu_ctx):
    gpu_ctx.set_precision("fp64")
    return gpu_ctx.prepare_superblock(conf("syn24"), 11)


def products(ctx, sb, n, prec):
    rng = np.random.default_rng(7)
    psi = rng.standard_normal(n)
    phi = rng.standard_normal(n)
    a, b = 0.7, -1.3
    ctx.set_precision(prec)
    try:
        hp = ctx.sigma(sb, psi)
        hf = ctx.sigma(sb, phi)
        hl = ctx.sigma(sb, a * psi + b * phi)
    finally:
        ctx.set_precision("fp64")
    return psi, phi, a, b, hp, hf, hl


@pytest.mark.parametrize("prec,tol", [("fp64", 1e-11), ("bf16x3tc", 2e-5)])
def test_hermitian_and_linear(gpu_ctx, big, prec, tol):
    sb, n = big
    assert n > 200000
    psi, phi, a, b, hp, hf, hl = products(gpu_ctx, sb, n, prec)
    sym = abs(phi @ hp - psi @ hf) / (np.linalg.norm(phi) * np.linalg.norm(hp))
    lin = np.linalg.norm(hl - (a * hp + b * hf)) / np.linalg.norm(hl)
    assert sym <= tol, (prec, sym)
    assert lin <= tol, (prec, lin)


def test_split_matches_fp64(gpu_ctx, big):
    sb, n = big
    _, _, _, _, hp64, _, _ = products(gpu_ctx, sb, n, "fp64")
    _, _, _, _, hp, _, _ = products(gpu_ctx, sb, n, "bf16x3tc")
    assert np.linalg.norm(hp - hp64) / np.linalg.norm(hp64) <= 2e-5
