"""Stacked stage-1 products of the tensor-core sigma (bgpu_set_tc_stacking):
products of small operator blocks that share a psi block run as one 128-row
MMA tile, each row sent to its own stage-1 operand.  Every row is the same
dot product as in the unstacked tile, so stacked and unstacked products
agree to rounding (1e-13 relative; both follow one summation order per
element), and both stay within the split tolerance (2e-5) of the FP64
oracle.  The D2h cases have many small sectors, so their plans hold stacks."""
import numpy as np
import pytest

from conftest import conf
from test_gpu_sigma import SNAPS, load

pytestmark = pytest.mark.gpu


@pytest.fixture
def tc_ctx(gpu_ctx):
    gpu_ctx.set_precision("bf16x3tc")
    yield gpu_ctx
    gpu_ctx.set_tc_stacking(64)
    gpu_ctx.set_tc_schedule(False)
    gpu_ctx.set_precision("fp64")


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("name,sweep,pos", SNAPS)
def test_stacked_matches_unstacked_and_oracle(tc_ctx, oracle, name, sweep, pos):
    snap = oracle.snapshot(conf(name), sweep, pos)
    sb, n = load(tc_ctx, snap)
    tc_ctx.set_tc_stacking(0)
    plain = tc_ctx.sigma(sb, snap["psi"])
    assert tc_ctx.superblock_info(sb)["tc_stacks"] == 0
    tc_ctx.set_tc_stacking(64)
    stacked = tc_ctx.sigma(sb, snap["psi"])
    info = tc_ctx.superblock_info(sb)
    if name == "c2_d2h":
        assert info["tc_stacks"] > 0 and info["tc_stacked_items"] >= 2 * info["tc_stacks"]
    assert rel(stacked, plain) <= 1e-13, (name, rel(stacked, plain))
    assert rel(stacked, snap["sigma"]) <= 2e-5
    assert np.array_equal(stacked, tc_ctx.sigma(sb, snap["psi"]))  # deterministic


@pytest.mark.parametrize("limit", [16, 128])
def test_stacking_limits_d2h(tc_ctx, limit):
    """A 20-orbital D2h superblock (many uneven sectors) at two stacking
    limits and in the per-sector baseline schedule, against FP64 and the
    unstacked product; stacking cuts the phase-1 tasks."""
    sb, n = tc_ctx.prepare_superblock(conf("syn20_d2h"), 9)
    rng = np.random.default_rng(5)
    psi = rng.standard_normal(n)
    tc_ctx.set_tc_stacking(0)
    plain = tc_ctx.sigma(sb, psi)
    tasks0 = tc_ctx.superblock_info(sb)["tc_phase1_tasks"]
    tc_ctx.set_tc_stacking(limit)
    stacked = tc_ctx.sigma(sb, psi)
    info = tc_ctx.superblock_info(sb)
    assert info["tc_stacks"] > 0
    assert info["tc_phase1_tasks"] < tasks0
    assert rel(stacked, plain) <= 1e-13
    tc_ctx.set_tc_schedule(True)
    per_sector = tc_ctx.sigma(sb, psi)
    tc_ctx.set_tc_schedule(False)
    assert rel(per_sector, plain) <= 1e-5
    tc_ctx.set_precision("fp64")
    ref = tc_ctx.sigma(sb, psi)
    tc_ctx.set_precision("bf16x3tc")
    assert rel(stacked, ref) <= 2e-5


def test_stacking_setting_checked(gpu_ctx):
    import block_gb300

    for bad in (-8, 12, 136):
        with pytest.raises(block_gb300.BgpuError):
            gpu_ctx.set_tc_stacking(bad)
    gpu_ctx.set_tc_stacking(64)
