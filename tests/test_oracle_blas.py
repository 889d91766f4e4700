"""The oracle's optional tuned DGEMM (the OpenBLAS bundled with SciPy, used
by the bench's CPU baseline as the reference links a BLAS): when a library
passes its child-process check, sigma matches the built-in loop to 1e-12
and the sweep still reproduces the reference's golden energy (1e-6 Eh)."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, conf


def test_blas_sigma_and_golden_energy(oracle):
    if not oracle.blas_candidates():
        pytest.skip("no SciPy-bundled OpenBLAS in this environment")
    ref = oracle.snapshot(conf("hubbard"), 1, 3)
    try:
        what = oracle.enable_blas()
        if "OpenBLAS" not in what:
            pytest.skip("the bundled OpenBLAS did not pass its check: " + what)
        got = oracle.snapshot(conf("hubbard"), 1, 3)
        assert np.linalg.norm(got["sigma"] - ref["sigma"]) <= 1e-12 * np.linalg.norm(ref["sigma"])
        e, _ = oracle.run(conf("hubbard"))
        with open(os.path.join(GOLDEN, "golden.json")) as f:
            gold = json.load(f)["hubbard"]
        for a, b in zip(e, gold["energies"]):
            assert abs(a - b) <= gold["tolerance"]
    finally:
        oracle.disable_blas()
