"""Output-tile widths of the tensor-core sigma (bgpu_set_tc_tile_width): 64
columns with two pipelines per SM and 128 columns with one, each against the
FP64 oracle within the split tolerance (2e-5 relative), and the two widths
against each other on the full-size 24-orbital M=500 superblock within 1e-5
(their sums differ only in how tiles split for load balance).  The
autotuner, which times both widths, records its choice in the plan."""
import numpy as np
import pytest

from conftest import conf
from test_gpu_sigma import SNAPS, load

pytestmark = pytest.mark.gpu


@pytest.fixture
def tc_ctx(gpu_ctx):
    gpu_ctx.set_precision("bf16x3tc")
    yield gpu_ctx
    gpu_ctx.set_tc_tile_width(0)
    gpu_ctx.set_autotune(False)
    gpu_ctx.set_precision("fp64")


@pytest.mark.parametrize("nb", [64, 128])
@pytest.mark.parametrize("name,sweep,pos", SNAPS)
def test_tile_width_matches_oracle(tc_ctx, oracle, nb, name, sweep, pos):
    snap = oracle.snapshot(conf(name), sweep, pos)
    sb, n = load(tc_ctx, snap)
    tc_ctx.set_tc_tile_width(nb)
    sig = tc_ctx.sigma(sb, snap["psi"])
    assert tc_ctx.superblock_info(sb)["tc_nb"] == nb
    err = np.linalg.norm(sig - snap["sigma"]) / np.linalg.norm(snap["sigma"])
    assert err <= 2e-5, (nb, name, err)
    assert np.array_equal(sig, tc_ctx.sigma(sb, snap["psi"]))  # deterministic


def test_widths_agree_full_size(tc_ctx):
    sb, n = tc_ctx.prepare_superblock(conf("syn24"), 11)
    rng = np.random.default_rng(3)
    psi = rng.standard_normal(n)
    out = {}
    for nb in (64, 128):
        tc_ctx.set_tc_tile_width(nb)
        out[nb] = tc_ctx.sigma(sb, psi)
        assert tc_ctx.superblock_info(sb)["tc_nb"] == nb
    tc_ctx.set_precision("fp64")
    ref = tc_ctx.sigma(sb, psi)
    for nb in (64, 128):
        assert np.linalg.norm(out[nb] - ref) / np.linalg.norm(ref) <= 2e-5
    assert np.linalg.norm(out[128] - out[64]) / np.linalg.norm(out[64]) <= 1e-5


def test_autotuner_chooses_a_width(tc_ctx, oracle):
    snap = oracle.snapshot(conf("c2_d2h"), 5, 5)
    sb, n = load(tc_ctx, snap)
    tc_ctx.set_autotune(True)
    sig = tc_ctx.sigma(sb, snap["psi"])
    info = tc_ctx.superblock_info(sb)
    assert info["tc_tuned"] == 1.0 and info["tc_nb"] in (64.0, 128.0)
    assert np.linalg.norm(sig - snap["sigma"]) / np.linalg.norm(snap["sigma"]) <= 2e-5
