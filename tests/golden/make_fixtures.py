"""Regenerates the golden fixtures of this directory from the reference tree.

Copies the FCIDUMP inputs of the reference's energy tests (data files only)
and records the expected energies its test scripts check:
  dmrg_tests/runtest:12,23,30,70 (test_energy.py tolerance 1e-6) and
  pydmrg/tests/test_dmrg_simple.py:34 (10 decimal places);
and copies the spatial one-particle density matrices its 1-RDM tests check
(dmrg_tests/runtest:31,141,152-154; test_onepdm.py and
test_transitiononepdm.py: sum of squared differences within 1e-7, the
transition matrix up to an overall sign).
Run where the reference tree is available, with its path as the required
argument (python make_fixtures.py <reference tree>); the tests read only
the committed copies.
"""
import hashlib
import json
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

CASES = {
    # name: (source FCIDUMP, conf body, expected energies, citation)
    "hubbard": ("dmrg_tests/hubbard/FCIDUMP",
                "nelec 8\nspin 0\nhf_occ integral\nschedule\n0 50 1.0e-6 0\n4 150 1e-6 0\n6 200 1e-6 0\n8 200 1e-8 0\nend\n"
                "maxiter 30\nsweep_tol 1e-9\nnroots 2\nweights 0.5 0.5\n",
                [-6.56819216], "dmrg_tests/runtest:30"),
    "pydmrg_fcidump1": ("pydmrg/tests/FCIDUMP-1",
                        "nelec 4\nspin 0\nirrep 1\nhf_occ integral\nschedule\n0 20 1.0e-6 0\n8 50 1e-8 0\n18 100 1e-8 0\nend\n"
                        "maxiter 30\nsweep_tol 1e-8\nsym d2h\n",
                        [-17.10516373008], "pydmrg/tests/test_dmrg_simple.py:34"),
    "c2_d2h": ("dmrg_tests/c2_d2h/FCIDUMP",
               "nelec 8\nspin 0\nirrep 1\nhf_occ integral\nschedule\n0 50 1.0e-6 0\n4 150 1e-6 0\n6 400 1e-6 0\n8 400 1e-10 0\nend\n"
               "maxiter 12\nsweep_tol 1e-9\nsym d2h\nnroots 2\nweights 0.5 0.5\n",
               [-75.4844085040, -74.9778423596], "dmrg_tests/runtest:12"),
    "h2o_nosym": ("dmrg_tests/h2o_nosym/FCIDUMP",
                  "nelec 10\nspin 0\nirrep 1\nhf_occ integral\nschedule default\nstartM 100\nmaxM 300\nsweep_tol tight\n",
                  [-76.11460447], "dmrg_tests/runtest:23"),
    # hubbard_stateSpecific/dmrg.conf (8-site ring, spin 6, 20 roots with
    # equal weights, state-averaged, perturbative noise in the first three
    # schedule entries) without twodot_to_onedot; davidson_max_iter lifts
    # this library's default limit (the reference's Davidson has none) so
    # that the degenerate top roots converge; the first 20 energies of the
    # runtest:70 list
    "hubbard_20roots": ("dmrg_tests/hubbard_stateSpecific/FCIDUMP",
                        "nelec 8\nspin 6\nhf_occ integral\nschedule\n0 50 1.0e-6 1e-06\n4 150 1e-6 1e-6\n"
                        "6 200 1e-6 1e-6\n8 200 1e-10 0.0\nend\nmaxiter 30\nsweep_tol 1e-9\nnroots 20\n"
                        "weights" + " 0.1" * 20 + "\ndavidson_max_iter 1000\n",
                        [-2.5065432138, -2.1684123422, -2.1684123422, -1.4755687956, -1.4755687956,
                         -1.4142135624, -1.4142135624, -1.2897006828, -0.8284271247, -0.5180081887,
                         -0.5180081887, -0.4079274397, -0.4079274397, 0.0, 0.0, 0.1224001196, 0.1224001196,
                         0.5857864376, 0.5857864376, 0.5857864376],
                        "dmrg_tests/runtest:70"),
    # h2o_transitionpdm/dmrg_onepdm.conf without its noise column and
    # twodot_to_onedot; no energy test in runtest (energies None)
    "h2o_c2v": ("dmrg_tests/h2o_transitionpdm/FCIDUMP",
                "nelec 10\nspin 0\nhf_occ integral\nschedule\n0 50 1.0e-6 0\n4 150 1e-6 0\n6 200 1e-6 0\n8 500 1e-8 0\nend\n"
                "maxiter 30\nsweep_tol 1e-9\nsym c2v\nirrep 1\nnroots 2\nweights 0.5 0.5\n",
                None, "dmrg_tests/runtest:149-154"),
}

# case: [(source, file name here, (bra, ket), citation)]; the hubbard root-1
# matrix comes from the transition test of the same FCIDUMP and schedule
ONEPDM = {
    "hubbard": [("dmrg_tests/hubbard/spat_onepdm.0.0.txt", "spat_onepdm.0.0.txt", (0, 0), "dmrg_tests/runtest:31"),
                ("dmrg_tests/hubbard_transition_pdm/spat_onepdm.1.1.txt", "spat_onepdm.1.1.txt", (1, 1),
                 "dmrg_tests/runtest:141")],
    "h2o_c2v": [("dmrg_tests/h2o_transitionpdm/spat_onepdm.0.0.txt", "spat_onepdm.0.0.txt", (0, 0),
                 "dmrg_tests/runtest:152"),
                ("dmrg_tests/h2o_transitionpdm/spat_onepdm.1.1.txt", "spat_onepdm.1.1.txt", (1, 1),
                 "dmrg_tests/runtest:153"),
                ("dmrg_tests/h2o_transitionpdm/spat_onepdm.1.0.txt", "spat_onepdm.1.0.txt", (1, 0),
                 "dmrg_tests/runtest:154")],
}


def main(argv):
    if len(argv) != 2:
        sys.exit("usage: python make_fixtures.py <path of the reference source tree>")
    ref = argv[1]
    meta = {}
    for name, (src, conf, energies, cite) in CASES.items():
        d = os.path.join(HERE, name)
        os.makedirs(d, exist_ok=True)
        shutil.copyfile(os.path.join(ref, src), os.path.join(d, "FCIDUMP"))
        with open(os.path.join(d, "dmrg.conf"), "w") as f:
            f.write(conf + "orbitals FCIDUMP\n")
        with open(os.path.join(d, "FCIDUMP"), "rb") as f:
            sha = hashlib.sha256(f.read()).hexdigest()
        meta[name] = dict(energies=energies, source=src, cited=cite, sha256=sha, tolerance=1e-6)
        pdms = []
        for psrc, dst, (bra, ket), pcite in ONEPDM.get(name, []):
            shutil.copyfile(os.path.join(ref, psrc), os.path.join(d, dst))
            with open(os.path.join(d, dst), "rb") as f:
                psha = hashlib.sha256(f.read()).hexdigest()
            pdms.append(dict(file=dst, bra=bra, ket=ket, source=psrc, cited=pcite, sha256=psha, sumsq=1e-7))
        if pdms:
            meta[name]["onepdm"] = pdms
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(meta, f, indent=1)


if __name__ == "__main__":
    main(sys.argv)
