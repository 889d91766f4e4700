"""Sweep checkpoints on the GPU engine through bgpu_run_dmrg: a run stopped
after two sweeps (`checkpoint`) and resumed (`restart`) ends with the same
energies as an uninterrupted run, in FP64 and in the split precision (the
blocks, their rotation records for the guess transform and the sweep
counters come back from the file; tolerance 1e-10 Eh)."""
import pytest

from test_checkpoint import make_conf

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec", ["fp64", "bf16x3tc"])
def test_gpu_restart_matches_uninterrupted(gpu_ctx, tmp_path, prec):
    gpu_ctx.set_precision(prec)
    try:
        e_full, st_full = gpu_ctx.run_dmrg(make_conf(tmp_path, "full.conf", 4))
        ck = tmp_path / "ck.bin"
        _, st2 = gpu_ctx.run_dmrg(make_conf(tmp_path, "part1.conf", 2, "checkpoint %s\n" % ck))
        assert ck.exists() and st2["sweeps"] == 2
        e4, st4 = gpu_ctx.run_dmrg(make_conf(tmp_path, "part2.conf", 4, "checkpoint %s\nrestart\n" % ck))
        assert st4["sweeps"] == st_full["sweeps"] == 4
        assert abs(e4[0] - e_full[0]) <= 1e-10, (e4[0], e_full[0])
        assert abs(st4["last_sweep_energy"] - st_full["last_sweep_energy"]) <= 1e-10
    finally:
        gpu_ctx.set_precision("fp64")
