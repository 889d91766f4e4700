"""Block spill on the GPU engine (bgpu_set_spill): a run whose idle blocks
live in host memory gives the energies of a run with every block on the
device (1e-10 Eh, FP64 and the split precision with transformed guesses),
copies blocks back to the device, and holds less operator-arena storage
at its peak."""
import pytest

from test_checkpoint import make_conf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "bf16x3tc"])
def test_gpu_spill_matches_resident(gpu_ctx, tmp_path, prec):
    gpu_ctx.set_precision(prec)
    try:
        e0, st0 = gpu_ctx.run_dmrg(make_conf(tmp_path, "plain.conf", 4))
        gpu_ctx.set_spill(True)
        e1, st1 = gpu_ctx.run_dmrg(make_conf(tmp_path, "spill.conf", 4))
    finally:
        gpu_ctx.set_spill(False)
        gpu_ctx.set_precision("fp64")
    assert st1["sweeps"] == st0["sweeps"] == 4
    assert abs(e1[0] - e0[0]) <= 1e-10, (e1[0], e0[0])
    for a, b in zip(st1["sweep_energies"], st0["sweep_energies"]):
        assert abs(a - b) <= 1e-10
    assert st0["spill_fetches"] == 0 and st1["spill_fetches"] > 0
    assert 0 < st1["peak_block_bytes"] < st0["peak_block_bytes"]
