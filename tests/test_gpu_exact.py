"""Exact-slice tensor-core products (BGPU_PREC_EXACT_TC): six balanced
base-128 digit slices per operand row, the 21 digit products accumulated
exactly in f32 TMEM and summed in FP64.  The representation error is about
2^-43 of each row's largest element, so sigma agrees with FP64 to about
1e-12 relative (observed 1.0e-12 on the first Hubbard snapshot).

Tolerances written here:
  - sigma against the FP64 oracle within 1e-11 relative on the oracle's
    snapshots, and bit-identical on a second call;
  - on the full-size 24-orbital M=500 superblock against the FP64 GPU
    product within 1e-11 relative;
  - split-precision Davidson with defect correction whose restart products
    are the exact ones (refinement mode 2): the FP64 squared residual of the
    returned vectors within the solve's tolerance (1e-10) and energies
    within 1e-10 Eh of the FP64 solve.
"""
import numpy as np
import pytest

from conftest import conf
from test_gpu_sigma import SNAPS, load

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.fixture
def exact_ctx(gpu_ctx):
    yield gpu_ctx
    gpu_ctx.set_precision("fp64")
    gpu_ctx.set_refinement("exact")


@pytest.mark.parametrize("name,sweep,pos", SNAPS)
def test_exact_sigma_matches_oracle(exact_ctx, oracle, name, sweep, pos):
    snap = oracle.snapshot(conf(name), sweep, pos)
    sb, n = load(exact_ctx, snap)
    exact_ctx.set_precision("exacttc")
    sig = exact_ctx.sigma(sb, snap["psi"])
    assert rel(sig, snap["sigma"]) <= 1e-11, rel(sig, snap["sigma"])
    assert np.array_equal(sig, exact_ctx.sigma(sb, snap["psi"]))


def test_exact_sigma_full_size(exact_ctx):
    sb, n = exact_ctx.prepare_superblock(conf("syn24"), 11)
    rng = np.random.default_rng(7)
    psi = rng.standard_normal(n)
    ref = exact_ctx.sigma(sb, psi)
    exact_ctx.set_precision("exacttc")
    sig = exact_ctx.sigma(sb, psi)
    assert rel(sig, ref) <= 1e-11, rel(sig, ref)


@pytest.mark.parametrize("name,sweep,pos", SNAPS[:3])
def test_exact_restart_products(exact_ctx, oracle, name, sweep, pos):
    snap = oracle.snapshot(conf(name), sweep, pos)
    sb, n = load(exact_ctx, snap)
    tol = 1e-10
    e64, _, _ = exact_ctx.davidson(sb, n, nroots=1, tol=tol)
    exact_ctx.set_precision("bf16x3tc")
    exact_ctx.set_refinement("exact")
    e, v, _ = exact_ctx.davidson(sb, n, nroots=1, tol=tol, vectors=True)
    assert exact_ctx.refinement_stats()[2]
    exact_ctx.set_precision("fp64")
    r = exact_ctx.sigma(sb, v[0]) - e[0] * v[0]
    assert r @ r <= tol, (name, r @ r)
    assert abs(e[0] - e64[0]) <= 1e-10, (name, e[0], e64[0])


@pytest.mark.parametrize("name,p", [("c2_d2h", 4), ("h2o_nosym", 5), ("hubbard12", 5)])
def test_exact_renormalisation(exact_ctx, oracle, name, p):
    """U^T O U of split-precision runs on the exact-slice kernels (the
    renormalisation of every operator block, MatrixRotate,
    MatrixBLAS.C:553-572) against the oracle's FP64 block within 1e-11 of
    its largest element; FP64 runs keep the FP64 pipe (1e-12)."""
    from test_gpu_blocks import case_of, density_and_rotations, rel_max

    c = case_of(oracle, name, p)
    big, sb, _, _, _ = density_and_rotations(exact_ctx, c, name)
    exact_ctx.set_precision("bf16x3tc")
    small, n, _ = exact_ctx.renormalise(big, c["kept"], c["small_keys"], rotations=c["rot"])
    got = exact_ctx.block_download(small, n)
    err = rel_max(got, c["small_arena"])
    assert err <= 1e-11, (name, err)
