"""Full two-site sweeps on the GPU (bgpu_run_dmrg) reproduce the reference's
golden energies (1e-6 Eh) and the CPU oracle's energies on the same input."""
import json
import os

import pytest

from conftest import GOLDEN, conf

pytestmark = pytest.mark.gpu

with open(os.path.join(GOLDEN, "golden.json")) as f:
    GOLD = json.load(f)


@pytest.mark.parametrize("name", ["hubbard", "pydmrg_fcidump1", "c2_d2h"])
def test_gpu_sweep_golden(gpu_ctx, name):
    e, st = gpu_ctx.run_dmrg(conf(name))
    for got, ref in zip(e, GOLD[name]["energies"]):
        assert abs(got - ref) <= GOLD[name]["tolerance"], (name, got, ref)
    assert st["sigma_calls"] > 0


def test_gpu_sweep_matches_oracle(gpu_ctx, oracle):
    c = conf("syn8_d2h")
    e_gpu, _ = gpu_ctx.run_dmrg(c)
    e_cpu, _ = oracle.run(c)
    assert abs(e_gpu[0] - e_cpu[0]) <= 1e-9, (e_gpu, e_cpu)
