"""The oracle's restatement of the TRANSFORM guess (CpuEngine::
transform_guess; GuessWave::transform_previous_wavefunction,
guess_wavefunction.C:526-620): sweeps started from the transformed previous
wavefunctions converge to the energies of sweeps started from unit vectors
(1e-8 Eh; the truncating c2_d2h case within the reference's 1e-6) with far
fewer sigma products; the rotations kept with each block survive a
checkpoint restart, and a spilled run stays bit-identical to a resident one
(one thread)."""
import numpy as np
import pytest

from conftest import conf
from test_checkpoint import make_conf


@pytest.mark.parametrize("name,tol", [("hubbard12", 1e-8), ("syn8_d2h", 1e-8), ("c2_d2h", 1e-6)])
def test_guess_fewer_products_same_energy(oracle, name, tol):
    e0, st0 = oracle.run(conf(name))
    e1, st1 = oracle.run(conf(name), guess=True)
    assert np.max(np.abs(e1 - e0)) <= tol, (name, e1, e0)
    assert st1["sigma_calls"] < 0.7 * st0["sigma_calls"], (st1["sigma_calls"], st0["sigma_calls"])


def test_guess_checkpoint_restart(oracle, tmp_path):
    e_full, st_full = oracle.run(make_conf(tmp_path, "full.conf", 4), guess=True, threads=1)
    ck = tmp_path / "ck.bin"
    oracle.run(make_conf(tmp_path, "part1.conf", 2, "checkpoint %s\n" % ck), guess=True, threads=1)
    e4, st4 = oracle.run(make_conf(tmp_path, "part2.conf", 4, "checkpoint %s\nrestart\n" % ck), guess=True,
                         threads=1)
    assert st4["sweeps"] == 4
    assert abs(e4[0] - e_full[0]) <= 1e-9
    assert np.array_equal(st4["sweep_energies"][2:], st_full["sweep_energies"][2:])


def test_guess_with_spill(oracle, tmp_path):
    e0, st0 = oracle.run(make_conf(tmp_path, "plain.conf", 4), guess=True, threads=1)
    e1, st1 = oracle.run(make_conf(tmp_path, "spill.conf", 4, "spill\n"), guess=True, threads=1)
    assert np.array_equal(e1, e0) and np.array_equal(st1["sweep_energies"], st0["sweep_energies"])
    assert st1["sigma_calls"] == st0["sigma_calls"] and st1["spill_fetches"] > 0
