"""The committed benchmark inputs are exactly what tests/golden/make_configs.py
writes (its CONFS table), so a change to one without the other shows up."""
import importlib.util
import os

from conftest import GOLDEN


def test_configs_match_their_generator():
    spec = importlib.util.spec_from_file_location("make_configs", os.path.join(GOLDEN, "make_configs.py"))
    mc = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mc)
    for name, (orb, body) in mc.CONFS.items():
        with open(os.path.join(GOLDEN, name, "dmrg.conf")) as f:
            assert f.read() == body + "orbitals %s\n" % orb, name
