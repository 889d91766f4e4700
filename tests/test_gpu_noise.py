"""Sweeps with density-matrix noise on the GPU: the schedule's perturbative
noise in the first two sweeps and twodot_noise's random noise in the first
(tests/golden/c2_d2h_noise).  Tolerances written here: the same seed gives
bit-identical sweep energies on a second run, and every sweep energy is
within 1e-7 Eh of the oracle's run of the same input (the noise terms are
summed in different orders on the two engines, which can move the
truncation by rounding)."""
import numpy as np
import pytest

from conftest import conf

pytestmark = pytest.mark.gpu


def test_noisy_sweeps_deterministic_and_match_oracle(gpu_ctx, oracle):
    e1, s1 = gpu_ctx.run_dmrg(conf("c2_d2h_noise"))
    e2, s2 = gpu_ctx.run_dmrg(conf("c2_d2h_noise"))
    assert np.array_equal(s1["sweep_energies"], s2["sweep_energies"]) and np.array_equal(e1, e2)
    eo, so = oracle.run(conf("c2_d2h_noise"))
    assert len(so["sweep_energies"]) == len(s1["sweep_energies"])
    for a, b in zip(s1["sweep_energies"], so["sweep_energies"]):
        assert abs(a - b) <= 1e-7, (a, b)
    # without noise the same schedule ends elsewhere in the first sweep
    e0, s0 = gpu_ctx.run_dmrg(conf("c2_d2h_m50"))
    assert abs(s0["sweep_energies"][0] - s1["sweep_energies"][0]) > 1e-4
