"""bench.py's `batching` entry on the CPU: the child run's command line is the
batching superblock's sigma measurement with its schedule comparisons and
without any recursion, its JSON line is reduced to the entry's fields, and a
child that fails leaves an `error` entry instead of failing the headline
line."""
import json
import subprocess
import sys
import types

from conftest import ROOT

CHILD_LINE = {
    "metric": "m", "value": 1.6, "ms_per_step": 3.6, "sigma_flops_per_step": 5.8e9, "prepare_seconds": 86.0,
    "config": {"workload": "batching superblock", "psi_elems": 62692},
    "e2e": {"value": 1.5}, "clocks": {"sm_mhz": 2070.0, "reasons": []},
    "roofline": {"tc_mma_issued_frac": 0.06, "tc_plan": {"tc_mma_flops": 4.3e11}},
    "schedules": {"per_sector": {"ms_per_sigma": 848.0}, "unstacked": {"ms_per_sigma": 7.8}},
    "fp64_path": {"ms_per_step": 390.0},
}


def _bench(monkeypatch):
    sys.path.insert(0, ROOT)
    monkeypatch.setattr(sys, "argv", ["bench.py"])
    import bench

    return bench


def test_batching_entry_from_child_line(monkeypatch):
    bench = _bench(monkeypatch)
    seen = {}

    def fake_run(cmd, **kw):
        seen["cmd"] = cmd
        return types.SimpleNamespace(stdout="log line\n" + json.dumps(CHILD_LINE) + "\n", returncode=0)

    monkeypatch.setattr(bench.subprocess, "run", fake_run)
    entry = bench.run_batching(bench.parse())
    cmd = seen["cmd"]
    assert cmd[cmd.index("--conf") + 1] == bench.BATCH_CONF and "--no-batching" in cmd
    for flag in ("--no-sweeps", "--no-exact", "--no-davidson"):
        assert flag in cmd
    assert "--no-schedules" not in cmd  # the per-sector and unstacked comparisons are the point
    assert entry["ms_per_sigma"] == 3.6 and entry["tflops"] == 1.6 and entry["psi_elems"] == 62692
    assert entry["schedules"]["per_sector"]["ms_per_sigma"] == 848.0
    assert entry["tc_mma_flops"] == 4.3e11


def test_batching_child_failure_is_recorded(monkeypatch):
    bench = _bench(monkeypatch)

    def fail(cmd, **kw):
        raise subprocess.TimeoutExpired(cmd, 900)

    monkeypatch.setattr(bench.subprocess, "run", fail)
    entry = bench.run_batching(bench.parse())
    assert "error" in entry and entry["conf"].endswith("syn30_d2h/dmrg.conf")
