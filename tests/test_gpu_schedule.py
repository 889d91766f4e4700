"""Schedules of the tensor-core sigma through the C ABI.

The per-sector baseline (one launch per psi / sigma sector, one block per
tile) and autotuned persistent schedules compute the same products as the
default persistent schedule: relative difference <= 1e-5 between schedules
(only the split-tile summation order differs), each within the split
tolerance 2e-5 of the FP64 oracle.  Tuned knobs are cached under the
superblock's sector-size histogram: a superblock with the same sectors reuses
them without timing, also from the cache file in a new context."""
import numpy as np
import pytest

from conftest import conf
from test_gpu_sigma import load

pytestmark = pytest.mark.gpu

KNOBS = ("tc_item_cost", "tc_split", "tc_group")


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture
def tc_ctx(gpu_ctx):
    gpu_ctx.set_precision("bf16x3tc")
    yield gpu_ctx
    gpu_ctx.set_tc_schedule(False)
    gpu_ctx.set_autotune(False)
    gpu_ctx.set_precision("fp64")


@pytest.mark.parametrize("name,sweep,pos", [("c2_d2h", 5, 5), ("pydmrg_fcidump1", 3, 4)])
def test_per_sector_schedule_matches(tc_ctx, oracle, name, sweep, pos):
    snap = oracle.snapshot(conf(name), sweep, pos)
    sb, n = load(tc_ctx, snap)
    a = tc_ctx.sigma(sb, snap["psi"])
    info_a = tc_ctx.superblock_info(sb)
    tc_ctx.set_tc_schedule(True)
    b = tc_ctx.sigma(sb, snap["psi"])
    info_b = tc_ctx.superblock_info(sb)
    assert info_a["tc_per_sector"] == 0 and info_b["tc_per_sector"] == 1
    assert info_b["launches"] > info_a["launches"]
    assert rel(a, snap["sigma"]) <= 2e-5 and rel(b, snap["sigma"]) <= 2e-5
    assert rel(b, a) <= 1e-5
    tc_ctx.set_tc_schedule(False)
    c = tc_ctx.sigma(sb, snap["psi"])
    assert np.array_equal(a, c)  # the default schedule again: bit-identical


def test_autotune_caches_by_histogram(tc_ctx, oracle, tmp_path):
    import block_gb300

    snap = oracle.snapshot(conf("c2_d2h"), 5, 5)
    cache = tmp_path / "tc_tune.txt"
    tc_ctx.set_autotune(True, str(cache))
    t0, _, _ = tc_ctx.autotune_stats()
    sb, n = load(tc_ctx, snap)
    a = tc_ctx.sigma(sb, snap["psi"])
    info = tc_ctx.superblock_info(sb)
    t1, c1, secs = tc_ctx.autotune_stats()
    assert info["tc_tuned"] == 1 and t1 == t0 + 1 and c1 >= 1 and secs > 0
    assert rel(a, snap["sigma"]) <= 2e-5
    # same sectors: knobs from the cache, no timing, same products
    sb2, _ = load(tc_ctx, snap)
    b = tc_ctx.sigma(sb2, snap["psi"])
    info2 = tc_ctx.superblock_info(sb2)
    t2, _, _ = tc_ctx.autotune_stats()
    assert t2 == t1 and info2["tc_tuned"] == 1
    assert all(info2[k] == info[k] for k in KNOBS)
    assert np.array_equal(a, b)
    # a new context reads the knobs from the cache file
    assert cache.read_text().count("\n") == 1
    ctx2 = block_gb300.Context(0)
    try:
        ctx2.set_precision("bf16x3tc")
        ctx2.set_autotune(True, str(cache))
        sb3, _ = load(ctx2, snap)
        c = ctx2.sigma(sb3, snap["psi"])
        tuned, cached, _ = ctx2.autotune_stats()
        assert tuned == 0 and cached == 1
        assert all(ctx2.superblock_info(sb3)[k] == info[k] for k in KNOBS)
        assert np.array_equal(a, c)
    finally:
        ctx2.close()
