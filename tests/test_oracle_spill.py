"""Block spill (`spill` keyword, SweepDriver::spill_idle / resident) on the
CPU oracle engine: stored blocks that the current step does not read live
in host memory only and are copied back when a step needs them.  On one
thread the oracle's sums have a fixed order, and a spilled run is
bit-identical to a resident one (with several threads two resident runs
already differ at 1e-8 Eh in an unconverged sweep); it copies blocks both
ways and holds less block storage at its peak.  Checkpoints written while
blocks are spilled restart to the energies of an uninterrupted run (1e-9 Eh,
several threads), and the one-particle density matrices are unchanged."""
import numpy as np

from test_checkpoint import make_conf


def test_spill_matches_resident(oracle, tmp_path):
    e0, st0 = oracle.run(make_conf(tmp_path, "plain.conf", 4), threads=1)
    e1, st1 = oracle.run(make_conf(tmp_path, "spill.conf", 4, "spill\n"), threads=1)
    assert st1["sweeps"] == st0["sweeps"] == 4
    assert np.array_equal(e1, e0)
    assert np.array_equal(st1["sweep_energies"], st0["sweep_energies"])
    assert st0["spill_fetches"] == 0 and st0["spill_bytes_down"] == 0
    assert st1["spill_fetches"] > 0 and st1["spill_bytes_up"] > 0 and st1["spill_bytes_down"] > 0
    assert 0 < st1["peak_block_bytes"] < st0["peak_block_bytes"]


def test_spill_checkpoint_restart(oracle, tmp_path):
    e_full, st_full = oracle.run(make_conf(tmp_path, "full.conf", 4))
    ck = tmp_path / "ck.bin"
    _, st2 = oracle.run(make_conf(tmp_path, "part1.conf", 2, "spill\ncheckpoint %s\n" % ck))
    assert ck.exists() and st2["sweeps"] == 2
    e4, st4 = oracle.run(make_conf(tmp_path, "part2.conf", 4, "spill\ncheckpoint %s\nrestart\n" % ck))
    assert st4["sweeps"] == 4
    assert abs(e4[0] - e_full[0]) <= 1e-9
    assert abs(st4["last_sweep_energy"] - st_full["last_sweep_energy"]) <= 1e-9


def test_spill_onepdm(oracle, tmp_path):
    oracle.run(make_conf(tmp_path, "plain.conf", 2, "onepdm\n"), threads=1)
    g0 = oracle.onepdm(0, 12)
    oracle.run(make_conf(tmp_path, "spill.conf", 2, "onepdm\nspill\n"), threads=1)
    g1 = oracle.onepdm(0, 12)
    assert np.array_equal(g1, g0)
