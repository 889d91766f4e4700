"""Sweep checkpoints (this project's restart format, host/checkpoint.h) on
the CPU oracle engine: a run stopped after two sweeps with `checkpoint` and
resumed with `restart` ends with the same energies and sweep count as an
uninterrupted run (to 1e-9 Eh: the oracle's OpenMP operator-pair sums are
not summed in a fixed order, so two runs of the same input differ at the
1e-11 level); `reset_iter` restarts the schedule; a
checkpoint refuses another Hamiltonian, and a truncated file is refused."""
import os

import pytest

from conftest import GOLDEN


def make_conf(tmp_path, name, maxiter, extra="", fcidump=None):
    src = os.path.join(GOLDEN, "hubbard12", "dmrg.conf")
    lines = []
    for l in open(src):
        if l.startswith("maxiter"):
            l = "maxiter %d\n" % maxiter
        if l.startswith("orbitals"):
            l = "orbitals %s\n" % (fcidump or os.path.join(GOLDEN, "hubbard12", "FCIDUMP"))
        lines.append(l)
    path = tmp_path / name
    path.write_text("".join(lines) + extra)
    return str(path)


def test_restart_matches_uninterrupted(oracle, tmp_path):
    e_full, st_full = oracle.run(make_conf(tmp_path, "full.conf", 4))
    ck = tmp_path / "ck.bin"
    e2, st2 = oracle.run(make_conf(tmp_path, "part1.conf", 2, "checkpoint %s\n" % ck))
    assert ck.exists() and st2["sweeps"] == 2
    e4, st4 = oracle.run(make_conf(tmp_path, "part2.conf", 4, "checkpoint %s\nrestart\n" % ck))
    assert st4["sweeps"] == st_full["sweeps"] == 4
    assert abs(e4[0] - e_full[0]) <= 1e-9, (e4[0], e_full[0])
    assert abs(st4["last_sweep_energy"] - st_full["last_sweep_energy"]) <= 1e-9


def test_reset_iter_restarts_schedule(oracle, tmp_path):
    ck = tmp_path / "ck.bin"
    oracle.run(make_conf(tmp_path, "part1.conf", 2, "checkpoint %s\n" % ck))
    e, st = oracle.run(make_conf(tmp_path, "again.conf", 2, "checkpoint %s\nrestart\nreset_iter\n" % ck))
    assert st["sweeps"] == 2  # the schedule ran from its first entry again
    e_full, _ = oracle.run(make_conf(tmp_path, "full.conf", 4))
    assert abs(e[0] - e_full[0]) <= 1e-6  # converged M=100 energy either way


def test_checkpoint_refuses_other_hamiltonian(oracle, tmp_path):
    ck = tmp_path / "ck.bin"
    oracle.run(make_conf(tmp_path, "part1.conf", 2, "checkpoint %s\n" % ck))
    # the same chain with U = 4.5 instead of 4
    dump = tmp_path / "FCIDUMP_u45"
    out = []
    for l in open(os.path.join(GOLDEN, "hubbard12", "FCIDUMP")):
        t = l.split()
        if len(t) == 5 and t[1] == t[2] == t[3] == t[4] and t[1] != "0":
            l = "%20.12f %4s %4s %4s %4s\n" % (4.5, t[1], t[2], t[3], t[4])
        out.append(l)
    dump.write_text("".join(out))
    with pytest.raises(RuntimeError):
        oracle.run(make_conf(tmp_path, "other.conf", 4, "checkpoint %s\nrestart\n" % ck, fcidump=str(dump)))


def test_truncated_checkpoint_refused(oracle, tmp_path):
    ck = tmp_path / "ck.bin"
    oracle.run(make_conf(tmp_path, "part1.conf", 2, "checkpoint %s\n" % ck))
    data = ck.read_bytes()
    ck.write_bytes(data[: len(data) // 2])
    with pytest.raises(RuntimeError):
        oracle.run(make_conf(tmp_path, "part2.conf", 4, "checkpoint %s\nrestart\n" % ck))
