"""bgpu_sigma_noalloc: sigma through the allocation-free entry point.

Some callers cannot let a library allocate device memory while they run
(work being recorded into a CUDA graph, a fixed device-memory budget, or an
application whose own allocator owns the GPU).  For them the library keeps
one fixed device array for the intermediates of the sigma product.  This
test checks, through the C ABI, that two consecutive allocation-free calls
give the same result as the regular device-buffer entry point (within the
1e-12 relative tolerance of the other sigma tests), and that a superblock
whose intermediates do not fit the array is refused with a clear error.
It sits in its own file named to be collected last.
"""
import numpy as np
import pytest

from conftest import conf

pytestmark = pytest.mark.gpu


def _superblock(ctx, snap):
    hl, _ = ctx.block_define(snap["orbsym"], snap["group"], snap["L"]["quanta"], snap["L"]["states"],
                             snap["L"]["keys"], snap["L"]["is_dot"])
    hr, _ = ctx.block_define(snap["orbsym"], snap["group"], snap["R"]["quanta"], snap["R"]["states"],
                             snap["R"]["keys"], snap["R"]["is_dot"])
    ctx.block_upload(hl, snap["L"]["arena"])
    ctx.block_upload(hr, snap["R"]["arena"])
    return ctx.superblock_define(hl, hr, snap["target"], snap["coef"], snap["ops"], snap["ecore"])


def test_noalloc_matches_device_entry_point(oracle):
    import block_gb300

    snap = oracle.snapshot(conf("c2_d2h"), 5, 5)
    with block_gb300.Context(0) as ctx:
        sb, n = _superblock(ctx, snap)
        x, y_ref, y_na = ctx.device_alloc(n), ctx.device_alloc(n), ctx.device_alloc(n)
        rng = np.random.default_rng(7)
        for call, psi in enumerate([snap["psi"], rng.standard_normal(n)]):
            ctx.to_device(x, psi)
            ctx.sigma_device(sb, x, y_ref)
            ctx.sigma_noalloc(sb, x, y_na)
            ctx.synchronize()
            ref = ctx.to_host(y_ref, n)
            got = ctx.to_host(y_na, n)
            err = np.linalg.norm(got - ref) / np.linalg.norm(ref)
            assert err <= 1e-12, (call, err)
            if call == 0:
                assert np.linalg.norm(got - snap["sigma"]) / np.linalg.norm(snap["sigma"]) <= 1e-12
        for p in (x, y_ref, y_na):
            ctx.device_free(p)


def test_noalloc_is_fp64_whatever_the_precision(oracle):
    """The allocation-free product is the FP64 one even after a split
    precision is chosen (its packed pools would need allocations)."""
    import block_gb300

    snap = oracle.snapshot(conf("c2_d2h"), 5, 5)
    with block_gb300.Context(0) as ctx:
        sb, n = _superblock(ctx, snap)
        x, y = ctx.device_alloc(n), ctx.device_alloc(n)
        ctx.to_device(x, snap["psi"])
        ctx.set_precision("bf16x3tc")
        for _ in range(2):
            ctx.sigma_noalloc(sb, x, y)
            ctx.synchronize()
            got = ctx.to_host(y, n)
            assert np.linalg.norm(got - snap["sigma"]) / np.linalg.norm(snap["sigma"]) <= 1e-12
        ctx.device_free(x)
        ctx.device_free(y)


def test_noalloc_rejects_oversized_superblock():
    import block_gb300

    with block_gb300.Context(0) as ctx:
        sb, n = ctx.prepare_superblock(conf("syn24"), 11)
        # the case is chosen because its FP64 intermediates exceed the array
        need = ctx.superblock_info(sb)["fp64_scratch"]
        assert need > block_gb300.NOALLOC_SCRATCH_DOUBLES, need
        x, y = ctx.device_alloc(n), ctx.device_alloc(n)
        with pytest.raises(block_gb300.BgpuError, match="more than the fixed"):
            ctx.sigma_noalloc(sb, x, y)
        ctx.device_free(x)
        ctx.device_free(y)
