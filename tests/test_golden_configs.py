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


def test_fixtures_match_their_recorded_hashes():
    """The FCIDUMPs and 1-RDM tables copied from the reference by
    make_fixtures.py are the files whose sha256 it recorded."""
    import hashlib
    import json

    with open(os.path.join(GOLDEN, "golden.json")) as f:
        gold = json.load(f)

    def sha(path):
        with open(path, "rb") as f:
            return hashlib.sha256(f.read()).hexdigest()

    n = 0
    for name, meta in gold.items():
        assert sha(os.path.join(GOLDEN, name, "FCIDUMP")) == meta["sha256"], name
        n += 1
        for pdm in meta.get("onepdm", []):
            assert sha(os.path.join(GOLDEN, name, pdm["file"])) == pdm["sha256"], (name, pdm["file"])
    assert n >= 5
