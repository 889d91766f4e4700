"""Oracle restatement of the density-matrix noise (CPU): the noise is
deterministic for a seed, changes the density matrix by about its
amplitude, and zero amplitudes leave it untouched."""
import numpy as np

from conftest import conf


def test_noise_deterministic_and_scaled(oracle):
    a = oracle.block_case(conf("c2_d2h"), 4)
    b = oracle.block_case(conf("c2_d2h"), 4, noise=1e-4, random_noise=1e-3, seed=7)
    b2 = oracle.block_case(conf("c2_d2h"), 4, noise=1e-4, random_noise=1e-3, seed=7)
    c = oracle.block_case(conf("c2_d2h"), 4, noise=1e-4, random_noise=1e-3, seed=8)
    z = oracle.block_case(conf("c2_d2h"), 4, noise=0.0, random_noise=0.0, seed=7)
    assert np.array_equal(b["rho"], b2["rho"])
    assert np.array_equal(z["rho"], a["rho"])
    assert not np.array_equal(b["rho"], c["rho"])  # another seed, other random vectors
    # the trace grows by the random amplitude plus the perturbative one
    # (each term is a unit-trace matrix times its amplitude)
    off = 0
    tr_a = tr_b = 0.0
    for d in a["big_states"]:
        tr_a += np.trace(a["rho"][off:off + d * d].reshape(d, d))
        tr_b += np.trace(b["rho"][off:off + d * d].reshape(d, d))
        off += d * d
    assert abs((tr_b - tr_a) - 1.1e-3) <= 1e-9, tr_b - tr_a
