"""The CPU oracle reproduces the reference's golden energies
(dmrg_tests/runtest, pydmrg/tests/test_dmrg_simple.py; tolerance 1e-6 Eh),
including the 20 state-averaged roots of the spin-3 Hubbard ring
(runtest:70), with their degenerate pairs and the four-fold level the
20th root falls into."""
import json
import os

import pytest

from conftest import GOLDEN, conf

with open(os.path.join(GOLDEN, "golden.json")) as f:
    GOLD = json.load(f)


@pytest.mark.parametrize("name", ["hubbard", "pydmrg_fcidump1", "c2_d2h", "h2o_nosym", "hubbard_20roots"])
def test_golden_energy(oracle, name):
    e, st = oracle.run(conf(name))
    want = GOLD[name]["energies"]
    assert len(e) >= len(want)
    for got, ref in zip(e, want):
        assert abs(got - ref) <= GOLD[name]["tolerance"], (name, got, ref)
