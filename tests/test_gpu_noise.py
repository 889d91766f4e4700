"""Sweeps with density-matrix noise on the GPU: the schedule's perturbative
noise in the first two sweeps and twodot_noise's random noise in the first
(tests/golden/syn16_noise: 16 orbitals, M=200, every step converged to
1e-12, unit-vector guesses as in the oracle).  Tolerances written here: the
same seed gives bit-identical sweep energies on a second run, and every
sweep energy is within 1e-6 Eh of the oracle's run of the same input (the
noise matrices themselves agree to 1e-13, tests/test_gpu_blocks.py; the
sweeps part by the Davidson tolerance's effect on an unconverged
trajectory, as without noise).  The random noise is drawn element by
element in the basis of the renormalised blocks, which the density-matrix
eigenvectors define: both engines make every eigenvector's largest
component positive, so that their bases, and with them the noise, agree."""
import numpy as np
import pytest

from conftest import conf

pytestmark = pytest.mark.gpu


def test_noisy_sweeps_deterministic_and_match_oracle(gpu_ctx, oracle):
    gpu_ctx.set_guess(False)
    try:
        e1, s1 = gpu_ctx.run_dmrg(conf("syn16_noise"))
        e2, s2 = gpu_ctx.run_dmrg(conf("syn16_noise"))
        e0, s0 = gpu_ctx.run_dmrg(conf("syn16_m200"))
    finally:
        gpu_ctx.set_guess(True)
    assert np.array_equal(s1["sweep_energies"], s2["sweep_energies"]) and np.array_equal(e1, e2)
    eo, so = oracle.run(conf("syn16_noise"))
    assert len(so["sweep_energies"]) == len(s1["sweep_energies"])
    for a, b in zip(s1["sweep_energies"], so["sweep_energies"]):
        assert abs(a - b) <= 1e-6, (a, b)
    # without noise the same schedule ends elsewhere in the first sweep
    assert abs(s0["sweep_energies"][0] - s1["sweep_energies"][0]) > 1e-5
