"""Element-wise parity, through the C ABI, of the operator work around sigma:
the enlarged-block build (bgpu_build_enlarged_ops: TensorProduct / Op::build,
operatorfunctions.C:146-254, Operators.C:453-2395), the density matrix and
its eigenvectors (bgpu_set_wavefunctions + bgpu_density_eig /
bgpu_density_download: makedensitymatrix, density.C:27-90; diagonalise_dm,
rotationmat.C:258-279) and the renormalisation (bgpu_renormalise:
renormalise_transform, BaseOperator.C:341-363; MatrixRotate,
MatrixBLAS.C:553-572), each against the oracle on the same inputs.

Tolerances written here: built operators and renormalised operators within
1e-12 of the oracle's relative to the largest element; the density matrix
within 1e-14 (absolute, its trace is 1); eigenvalues within 1e-12; each
eigenvector of a nondegenerate eigenvalue (relative gap above 1e-6) equal to
the oracle's up to its sign within 1e-9 (eigenvalues of a sector closer than
1e-6 of the sector's largest are degenerate for this check: the eigenvectors
of a cluster are determined only as a subspace).
"""
import numpy as np
import pytest

from conftest import conf

pytestmark = pytest.mark.gpu

# (configuration, partition): the sector sizes reach 25, 8, 53 and 138 states,
# so both the small-sector and the large-sector eigensolvers run
CASES = [("c2_d2h", 4), ("syn8_d2h", 3), ("hubbard12", 5), ("h2o_nosym", 5), ("syn24_m250", 5)]

_cache = {}


def case_of(oracle, name, p):
    if (name, p) not in _cache:
        _cache[(name, p)] = oracle.block_case(conf(name), p)
    return _cache[(name, p)]


def define(ctx, c, which, is_dot=False, keys=True):
    h, n = ctx.block_define(c["orbsym"], c["group"], c[which + "_quanta"], c[which + "_states"],
                            c[which + "_keys"] if keys else np.zeros((0, 4), np.int32), is_dot)
    ctx.block_set_sites(h, c[which + "_sites"])
    return h, n


def rel_max(got, ref):
    return float(np.max(np.abs(got - ref)) / max(np.max(np.abs(ref)), 1e-300))


def build_big(ctx, c, name):
    ints, norb = ctx.integrals_load(conf(name))
    assert norb == len(c["orbsym"])
    hs, ns = define(ctx, c, "sys")
    ctx.block_upload(hs, c["sys_arena"])
    hd, nd = define(ctx, c, "dot", is_dot=True)
    ctx.block_upload(hd, c["dot_arena"])
    big, n, nq = ctx.build_enlarged_ops(ints, hs, hd, c["big_keys"], filt=c["filter"])
    return big, n, nq


@pytest.mark.parametrize("name,p", CASES)
def test_build_enlarged_ops_matches_oracle(gpu_ctx, oracle, name, p):
    c = case_of(oracle, name, p)
    big, n, nq = build_big(gpu_ctx, c, name)
    q, st = gpu_ctx.block_quanta(big)
    assert nq == len(c["big_states"])
    np.testing.assert_array_equal(q, c["big_quanta"])
    np.testing.assert_array_equal(st, c["big_states"])
    assert n == c["big_arena"].size
    got = gpu_ctx.block_download(big, n)
    assert rel_max(got, c["big_arena"]) <= 1e-12, (name, rel_max(got, c["big_arena"]))


def density_and_rotations(ctx, c, name):
    big, n, nq = build_big(ctx, c, name)
    he, _ = define(ctx, c, "env", keys=False)
    sb, npsi = ctx.superblock_define(big, he, c["target"], np.zeros(0), np.zeros((0, 4), np.int32), 0.0)
    assert npsi == c["psi"].size
    ctx.set_wavefunctions(sb, c["psi"])
    eig = ctx.density_eig(sb, True, int(c["big_states"].sum()), [1.0])
    rho, vecs = ctx.density_download(c["rho"].size)
    return big, sb, eig, rho, vecs


@pytest.mark.parametrize("name,p", CASES)
def test_density_matrix_and_eigenpairs(gpu_ctx, oracle, name, p):
    c = case_of(oracle, name, p)
    _, _, eig, rho, vecs = density_and_rotations(gpu_ctx, c, name)
    assert np.max(np.abs(rho - c["rho"])) <= 1e-14
    assert np.max(np.abs(eig - c["eig"])) <= 1e-12
    off = 0
    e_off = 0
    for d in c["big_states"]:
        V = vecs[off:off + d * d].reshape(d, d)
        R = c["vecs"][off:off + d * d].reshape(d, d)
        w = c["eig"][e_off:e_off + d]
        wmax = max(np.max(np.abs(w)), 1e-300)
        for j in range(d):
            gaps = np.abs(np.delete(w, j) - w[j]) if d > 1 else np.array([np.inf])
            if gaps.min() <= 1e-6 * wmax:
                continue  # degenerate: any basis of the eigenspace is right
            s = np.sign(V[:, j] @ R[:, j])
            assert np.max(np.abs(s * V[:, j] - R[:, j])) <= 1e-9, (name, d, j)
        off += d * d
        e_off += d


@pytest.mark.parametrize("name,p", CASES)
def test_renormalise_matches_oracle(gpu_ctx, oracle, name, p):
    c = case_of(oracle, name, p)
    big, sb, _, _, _ = density_and_rotations(gpu_ctx, c, name)
    # the oracle's rotation, passed in
    small, n, nq = gpu_ctx.renormalise(big, c["kept"], c["small_keys"], rotations=c["rot"])
    q, st = gpu_ctx.block_quanta(small)
    np.testing.assert_array_equal(q, c["small_quanta"])
    np.testing.assert_array_equal(st, c["small_states"])
    got = gpu_ctx.block_download(small, n)
    assert rel_max(got, c["small_arena"]) <= 1e-12, (name, rel_max(got, c["small_arena"]))
    np.testing.assert_array_equal(gpu_ctx.rotation_download(small, c["rot"].size), c["rot"])
    # the GPU's own eigenvectors (never leaving the device) span the oracle's
    # kept space, and renormalising with them downloaded and passed back in
    # gives the same block
    small2, n2, _ = gpu_ctx.renormalise(big, c["kept"], c["small_keys"])
    rot = gpu_ctx.rotation_download(small2, c["rot"].size)
    off = 0
    for d, m in zip(c["big_states"], c["kept"]):
        if m:
            U = rot[off:off + d * m].reshape(d, m)
            R = c["rot"][off:off + d * m].reshape(d, m)
            s = np.linalg.svd(U.T @ R, compute_uv=False)
            assert np.max(np.abs(s - 1.0)) <= 1e-9, (name, d, m)
            off += d * m
    a = gpu_ctx.block_download(small2, n2)
    small3, n3, _ = gpu_ctx.renormalise(big, c["kept"], c["small_keys"], rotations=rot)
    b = gpu_ctx.block_download(small3, n3)
    assert rel_max(a, b) <= 1e-14


def test_boundary_errors(oracle):
    import block_gb300

    c = case_of(oracle, "syn8_d2h", 3)
    with block_gb300.Context(0) as ctx:
        boundary_errors(ctx, c)


def boundary_errors(gpu_ctx, c):
    import block_gb300

    ints, _ = gpu_ctx.integrals_load(conf("syn8_d2h"))
    hs, _ = gpu_ctx.block_define(c["orbsym"], c["group"], c["sys_quanta"], c["sys_states"], c["sys_keys"])
    hd, _ = define(gpu_ctx, c, "dot", is_dot=True)
    with pytest.raises(block_gb300.BgpuError, match="sites"):
        gpu_ctx.build_enlarged_ops(ints, hs, hd, c["big_keys"], filt=c["filter"])
    gpu_ctx.block_set_sites(hs, c["sys_sites"])
    with pytest.raises(block_gb300.BgpuError, match="operators"):
        gpu_ctx.build_enlarged_ops(ints, hs, hd, c["big_keys"], filt=c["filter"])
    gpu_ctx.block_upload(hs, c["sys_arena"])
    gpu_ctx.block_upload(hd, c["dot_arena"])
    # a catalogue the sub-blocks cannot build
    bad = np.array([[1, 7, -1, 1]], dtype=np.int32)  # C_7, a site outside both sub-blocks
    with pytest.raises(block_gb300.BgpuError, match="needs"):
        gpu_ctx.build_enlarged_ops(ints, hs, hd, bad, filt=c["filter"])
    big, _, nq = gpu_ctx.build_enlarged_ops(ints, hs, hd, c["big_keys"], filt=c["filter"])
    with pytest.raises(block_gb300.BgpuError, match="density"):
        gpu_ctx.renormalise(big, np.ones(nq, np.int32), c["small_keys"])
    gpu_ctx.integrals_free(ints)
    with pytest.raises(block_gb300.BgpuError, match="integrals"):
        gpu_ctx.build_enlarged_ops(ints, hs, hd, c["big_keys"], filt=c["filter"])


@pytest.mark.parametrize("name,p", [("c2_d2h", 4), ("h2o_nosym", 5), ("hubbard12", 5)])
def test_density_noise_matches_oracle(gpu_ctx, oracle, name, p):
    """Perturbative (add_onedot_noise) and random (add_twodot_noise) noise
    of the density matrix against the oracle's for the same wavefunction
    and seed: the noisy rho within 1e-13, its eigenvalues within 1e-12, and
    the same seed gives the same matrix on a second call."""
    c = oracle.block_case(conf(name), p, noise=1e-4, random_noise=1e-3, seed=7)
    gpu_ctx.set_density_noise(1e-4, 1e-3, 7)
    try:
        _, _, eig, rho, _ = density_and_rotations(gpu_ctx, c, name)
        _, _, eig2, rho2, _ = density_and_rotations(gpu_ctx, c, name)
    finally:
        gpu_ctx.set_density_noise(0.0, 0.0, 0)
    plain = case_of(oracle, name, p)
    assert np.max(np.abs(c["rho"] - plain["rho"])) > 1e-7  # the noise is there
    assert np.max(np.abs(rho - c["rho"])) <= 1e-13, np.max(np.abs(rho - c["rho"]))
    assert np.max(np.abs(eig - c["eig"])) <= 1e-12
    assert np.array_equal(rho, rho2) and np.array_equal(eig, eig2)
