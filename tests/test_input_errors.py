"""Host-side failure detection on the CPU: malformed dmrg.conf inputs, a
missing FCIDUMP, keywords of methods outside this path, and a restart
without a checkpoint are refused with an error (the reference aborts on
most of these, input.C; here the driver raises and the C ABI returns a
status code).  The parser and driver are the product's own host code; the
oracle engine runs them without a GPU."""
import os

import pytest

from conftest import GOLDEN

BASE = """nelec 12
spin 0
schedule
0 50 1e-8 0
end
maxiter 2
sweep_tol 1e-12
noreorder
orbitals {orb}
"""
FCIDUMP = os.path.join(GOLDEN, "hubbard12", "FCIDUMP")


def run_conf(oracle, tmp_path, text):
    p = tmp_path / "dmrg.conf"
    p.write_text(text)
    return oracle.run(str(p))


def test_valid_input_runs(oracle, tmp_path):
    e, st = run_conf(oracle, tmp_path, BASE.format(orb=FCIDUMP))
    assert st["sweeps"] == 2 and -7.0 < e[0] < -5.0


@pytest.mark.parametrize("text", [
    BASE.replace("0 50 1e-8 0", "0 50 1e-8"),                 # schedule line with 3 entries
    BASE.replace("schedule\n0 50 1e-8 0\nend\n", ""),        # no schedule
    BASE + "hubbard\n",                                        # other Hamiltonian family
    BASE + "onedot\n",                                         # one-site sweeps
    BASE + "nonspinadapted\n",                                 # determinant basis
    BASE.replace("maxiter 2", "maxiter"),                      # keyword without its value
    BASE.replace("orbitals {orb}", "orbitals synthetic:0:0:0:0:0"),  # empty synthetic system
    BASE + "davidson_max_iter 0\n",                          # iteration limit must be positive
    BASE + "davidson_max_iter\n",                            # ... and given
], ids=["schedule-entries", "no-schedule", "hubbard", "onedot", "nonspinadapted", "no-value", "bad-synthetic",
        "max-iter-zero", "max-iter-missing"])
def test_malformed_input_refused(oracle, tmp_path, text):
    with pytest.raises(RuntimeError):
        run_conf(oracle, tmp_path, text.format(orb=FCIDUMP))


def test_davidson_max_iter_limits_the_solves(oracle, tmp_path):
    """davidson_max_iter caps every solve: with one iteration per solve the
    sweep still runs (each step keeps its best Ritz vector) and stays above
    the converged energy."""
    e_ref, _ = run_conf(oracle, tmp_path, BASE.format(orb=FCIDUMP))
    e1, st1 = run_conf(oracle, tmp_path, BASE.format(orb=FCIDUMP) + "davidson_max_iter 1\n")
    assert st1["sweeps"] == 2 and e1[0] > e_ref[0] + 1e-6


def test_missing_fcidump_refused(oracle, tmp_path):
    with pytest.raises(RuntimeError):
        run_conf(oracle, tmp_path, BASE.format(orb=str(tmp_path / "no_such_FCIDUMP")))


def test_restart_without_checkpoint_refused(oracle, tmp_path):
    with pytest.raises(RuntimeError):
        run_conf(oracle, tmp_path, BASE.format(orb=FCIDUMP) + "restart\n")


def _dump(tmp_path, name, body_lines, norb=12):
    src = open(FCIDUMP).read().splitlines()
    head = []
    for l in src:
        head.append(l)
        if "&END" in l.upper() or l.strip() == "/":
            break
    p = tmp_path / name
    p.write_text("\n".join(head + body_lines) + "\n")
    return str(p)


def _integral_lines():
    lines = open(FCIDUMP).read().splitlines()
    k = next(i for i, l in enumerate(lines) if "&END" in l.upper() or l.strip() == "/")
    return lines[k + 1:]


def test_fcidump_fortran_exponents_and_comments(oracle, tmp_path):
    e_ref, _ = run_conf(oracle, tmp_path, BASE.format(orb=FCIDUMP))
    body = ["! integrals written with Fortran D exponents"]
    for l in _integral_lines():
        t = l.split()
        if len(t) == 5:
            body.append("%.15D %s %s %s %s".replace("%.15D", "%sD+00" % repr(float(t[0]))) % tuple(t[1:]))
    e, _ = run_conf(oracle, tmp_path, BASE.format(orb=_dump(tmp_path, "FCIDUMP_D", body)))
    assert abs(e[0] - e_ref[0]) <= 1e-9


@pytest.mark.parametrize("line", ["1.0 13 1 0 0", "1.0 1 1 1", "1.0x 1 1 0 0", "1.0 0 1 0 0", "1.0 1 2 0 3"],
                         ids=["index-above-norb", "four-fields", "bad-value", "orbital-0-one-electron",
                              "orbital-0-two-electron"])
def test_fcidump_bad_integral_line_refused(oracle, tmp_path, line):
    body = _integral_lines()
    body.insert(3, line)
    with pytest.raises(RuntimeError):
        run_conf(oracle, tmp_path, BASE.format(orb=_dump(tmp_path, "FCIDUMP_bad", body)))
