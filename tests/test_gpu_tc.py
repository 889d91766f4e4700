"""tcgen05 tile primitive: shared-memory operand layout, descriptors, TMEM
accumulation and read-back against a host product of the same bf16 values."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _bf16(rng, shape):
    x = rng.standard_normal(shape).astype(np.float32)
    bits = (x.view(np.uint32) >> 16).astype(np.uint16)
    vals = (bits.astype(np.uint32) << 16).view(np.float32)
    return bits, vals.astype(np.float64)


@pytest.mark.parametrize("n,k,packed", [(16, 16, False), (48, 16, False), (64, 64, False), (128, 32, False),
                                         (256, 64, False), (16, 16, True), (48, 80, True), (128, 128, True),
                                         (256, 256, True)])
def test_tc_tile_matches_host_product(gpu_ctx, n, k, packed):
    rng = np.random.default_rng(1000 + n + k)
    a_bits, a = _bf16(rng, (128, k))
    b_bits, b = _bf16(rng, (n, k))
    d = gpu_ctx.tc_tile(a_bits, b_bits, packed=packed)
    ref = a @ b.T
    # f32 accumulation of k exact bf16 x bf16 products
    err = np.abs(d - ref).max() / np.abs(ref).max()
    assert err < 1e-6, err


def test_bounded_wait_gives_up_and_reports(gpu_ctx):
    """The pipeline wait of the tensor-core kernels, on a barrier nothing
    arrives at, returns failure after its limit and sets the status word
    (the host-side check that turns it into an error); the context stays
    usable afterwards."""
    gave_up, status, waited = gpu_ctx.tc_wait_selftest(20.0)
    assert gave_up == 1 and status == 1
    assert 19.0 <= waited < 1000.0, waited
    a_bits = np.zeros((128, 16), dtype=np.uint16)
    b_bits = np.zeros((16, 16), dtype=np.uint16)
    assert np.all(gpu_ctx.tc_tile(a_bits, b_bits) == 0.0)
