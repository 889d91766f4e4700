"""sigma = H psi, diag(H) and Davidson of the CUDA library against the CPU
oracle on the same superblocks, through the C ABI (FP64 path: relative
sigma error <= 1e-12)."""
import numpy as np
import pytest

from conftest import conf

pytestmark = pytest.mark.gpu

SNAPS = [
    ("hubbard", 1, 3),
    ("hubbard", 2, 2),
    ("pydmrg_fcidump1", 3, 4),
    ("c2_d2h", 5, 5),
]


def load(ctx, snap):
    hl, _ = ctx.block_define(snap["orbsym"], snap["group"], snap["L"]["quanta"], snap["L"]["states"],
                             snap["L"]["keys"], snap["L"]["is_dot"])
    hr, _ = ctx.block_define(snap["orbsym"], snap["group"], snap["R"]["quanta"], snap["R"]["states"],
                             snap["R"]["keys"], snap["R"]["is_dot"])
    ctx.block_upload(hl, snap["L"]["arena"])
    ctx.block_upload(hr, snap["R"]["arena"])
    sb, n = ctx.superblock_define(hl, hr, snap["target"], snap["coef"], snap["ops"], snap["ecore"])
    assert n == snap["psi"].size
    return sb, n


@pytest.mark.parametrize("name,sweep,pos", SNAPS)
def test_sigma_matches_oracle(gpu_ctx, oracle, name, sweep, pos):
    snap = oracle.snapshot(conf(name), sweep, pos)
    sb, n = load(gpu_ctx, snap)
    sig = gpu_ctx.sigma(sb, snap["psi"])
    err = np.linalg.norm(sig - snap["sigma"]) / np.linalg.norm(snap["sigma"])
    assert err <= 1e-12, err
    d = gpu_ctx.hdiag(sb, n)
    assert np.max(np.abs(d - snap["diag"])) <= 1e-11 * max(1.0, np.max(np.abs(snap["diag"])))
    # deterministic: a second call is bit-identical
    sig2 = gpu_ctx.sigma(sb, snap["psi"])
    assert np.array_equal(sig, sig2)


@pytest.mark.parametrize("name,sweep,pos", SNAPS[:3])
def test_davidson_matches_dense(gpu_ctx, oracle, name, sweep, pos):
    snap = oracle.snapshot(conf(name), sweep, pos)
    sb, n = load(gpu_ctx, snap)
    assert n <= 2000
    # dense H column by column through the (oracle-checked) sigma product
    H = np.empty((n, n))
    eye = np.eye(n)
    for j in range(n):
        H[:, j] = gpu_ctx.sigma(sb, eye[j])
    assert np.max(np.abs(H - H.T)) <= 1e-11 * np.max(np.abs(H))
    w = np.linalg.eigvalsh(0.5 * (H + H.T))
    e, v, it = gpu_ctx.davidson(sb, n, nroots=1, tol=1e-14, vectors=True)
    assert abs(e[0] - w[0]) <= 1e-10, (e[0], w[0])
    # the oracle's wavefunction (converged to its sweep's Davidson tolerance) lies above
    assert snap["energy"] >= w[0] - 1e-10
    r = gpu_ctx.sigma(sb, v[0]) - e[0] * v[0]
    assert np.dot(r, r) <= 1e-12


@pytest.mark.parametrize("prec", ["fp64", "bf16x3tc"])
def test_davidson_graph_roots(gpu_ctx, oracle, prec):
    """Three roots through the device-resident Davidson: the captured-graph
    iteration and the same launches issued one by one give identical
    energies and iteration counts, and the roots match dense
    diagonalisation (the split path after its FP64 Rayleigh refinement)."""
    snap = oracle.snapshot(conf("hubbard"), 1, 3)
    sb, n = load(gpu_ctx, snap)
    H = np.empty((n, n))
    eye = np.eye(n)
    gpu_ctx.set_precision("fp64")
    for j in range(n):
        H[:, j] = gpu_ctx.sigma(sb, eye[j])
    w = np.linalg.eigvalsh(0.5 * (H + H.T))
    gpu_ctx.set_precision(prec)
    try:
        out = {}
        for graph in (True, False):
            gpu_ctx.set_davidson_graph(graph)
            e, v, it = gpu_ctx.davidson(sb, n, nroots=3, tol=1e-12 if prec == "fp64" else 1e-9, vectors=True)
            out[graph] = (e, v, it, gpu_ctx.davidson_graph_launches())
        assert out[True][3] > 0 and out[False][3] == 0
        assert out[True][2] == out[False][2]
        assert np.array_equal(out[True][0], out[False][0])
        assert np.array_equal(out[True][1], out[False][1])
        e = out[True][0]
        tol = 1e-9 if prec == "fp64" else 1e-8
        assert np.max(np.abs(e - w[:3])) <= tol, (e, w[:3])
    finally:
        gpu_ctx.set_davidson_graph(True)
        gpu_ctx.set_precision("fp64")
