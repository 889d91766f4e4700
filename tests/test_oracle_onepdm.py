"""The oracle's one-particle density matrix sweep (the onepdm keyword;
modules/onepdm/onepdm.C) against an independent determinant FCI in numpy:
gamma_pq = <Psi|E_pq|Psi> of the FCI eigenvector whose energy the DMRG run
reached, with E_pq the spin-summed excitation operator.

Tolerances written here: the DMRG solves converge the squared residual to
1e-12, so the wavefunction, and with it gamma, is exact to about 1e-7; the
test allows 1e-6 elementwise and 1e-6 on the trace (the electron count).
The cases cover C1 and D2h integrals, a singlet and a triplet (E_pq is a
spin scalar, so the M_S = 0 member of the FCI multiplet gives the same
gamma), a run whose orbitals the sweep reorders, with gamma reported in
the input orbital order (save_onepdm_spatial_text, onepdm.C:504-528), and
the two state-averaged roots of the 8-site Hubbard case with its final
Davidson tolerance tightened to 1e-12 (one gamma per root, 2e-6: the
second root's solve ends with a larger residual, observed 7e-7), and their
transition matrices <1|E_pq|0> and <0|E_pq|1> up to one overall sign
(elements from different sweep steps share the roots' relative phase).

The reference's own tables pin the same sweep: its 8-site Hubbard roots 0
and 1 and its C2v water roots 0, 1 and their transition matrix <1|E_kl|0>
(dmrg_tests/runtest:31,141,152-154) within the reference's measure, the sum
of squared differences at most 1e-7 (observed 8.5e-10, 1.9e-11, 8.3e-9 and
3.4e-8 for the water matrices and the Hubbard root 0)."""
import json
import os

import numpy as np
import pytest
import scipy.sparse.linalg as sla

from conftest import GOLDEN
from test_oracle_fci import fci_operators, write_fcidump


def fci_onepdm(t, v, ecore, nelec, energy, nroots=40, ket_energy=None):
    """<bra|E_pq|ket> of the FCI eigenvectors at the given energies (ket =
    bra without ket_energy)."""
    H, E = fci_operators(t, v, ecore, nelec)
    w, X = sla.eigsh(H, k=nroots, which="SA", tol=1e-13)

    def state(en):
        k = int(np.argmin(np.abs(w - en)))
        assert abs(w[k] - en) <= 1e-8, (w[k], en)
        assert np.min(np.abs(np.delete(w, k) - w[k])) > 1e-6  # a non-degenerate state
        return X[:, k]

    x = state(energy)
    y = x if ket_energy is None else state(ket_energy)
    n = t.shape[0]
    return np.array([[x @ (E[p, q] @ y) for q in range(n)] for p in range(n)])


def read_spatial_onepdm(path):
    with open(path) as f:
        n = int(f.readline())
        g = np.zeros((n, n))
        for line in f:
            i, j, x = line.split()
            g[int(i), int(j)] = float(x)
    return g


def onepdm_conf(tmp_path, name, spin=0, reorder=False):
    """The golden configuration with the onepdm keyword and the output
    prefix; its FCIDUMP (if any) by absolute path; the Hubbard case's final
    Davidson tolerance at 1e-12."""
    d = os.path.join(GOLDEN, name)
    body = open(os.path.join(d, "dmrg.conf")).read().replace("spin 0", "spin %d" % spin)
    body = body.replace("orbitals FCIDUMP", "orbitals %s" % os.path.join(d, "FCIDUMP"))
    body = body.replace("8 200 1e-8 0", "8 200 1e-12 0")
    if reorder:
        body = body.replace("noreorder\n", "")
    conf = tmp_path / "dmrg.conf"
    conf.write_text(body + "onepdm\nprefix %s\n" % tmp_path)
    return str(conf)


CASES = [
    ("syn8", 0, False, 1e-6),
    ("syn8_d2h", 0, False, 1e-6),
    ("syn8", 2, False, 1e-6),
    ("syn8", 0, True, 1e-6),
    ("hubbard", 0, False, 2e-6),
]


@pytest.mark.parametrize("name,spin,reorder,tol", CASES)
def test_onepdm_matches_fci(oracle, tmp_path, name, spin, reorder, tol):
    conf = onepdm_conf(tmp_path, name, spin, reorder)
    t, v, ecore = write_fcidump(oracle, conf, str(tmp_path / "FCIDUMP"), input_order=True)
    e, _ = oracle.run(conf)
    for r in range(len(e)):
        g = oracle.onepdm(r, 8)
        gf = fci_onepdm(t, v, ecore, 8, e[r])
        assert np.max(np.abs(g - gf)) <= tol, (r, np.max(np.abs(g - gf)))
        assert abs(np.trace(g) - 8) <= tol
        assert np.array_equal(g, g.T)
        # the text file holds the same matrix
        gt = read_spatial_onepdm(tmp_path / ("spatial_onepdm.%d.%d.txt" % (r, r)))
        assert np.max(np.abs(gt - g)) <= 1e-13 * np.max(np.abs(g))
    if len(e) > 1:
        # transition matrices: one relative sign of the two roots for all
        # elements, however many sweep steps they come from
        gf = fci_onepdm(t, v, ecore, 8, e[1], ket_energy=e[0])
        for a, b, ref in ((1, 0, gf), (0, 1, gf.T)):
            g = oracle.transition_onepdm(a, b, 8)
            d = min(np.max(np.abs(g - ref)), np.max(np.abs(g + ref)))
            assert d <= tol, (a, b, d)


def test_onepdm_needs_the_keyword(oracle):
    oracle.run(os.path.join(GOLDEN, "syn8", "dmrg.conf"))
    with pytest.raises(RuntimeError):
        oracle.onepdm(0, 8)


def golden_onepdm_cases():
    with open(os.path.join(GOLDEN, "golden.json")) as f:
        meta = json.load(f)
    return [(name, m["onepdm"]) for name, m in meta.items() if "onepdm" in m]


def onepdm_golden_conf(tmp_path, name, keyword):
    d = os.path.join(GOLDEN, name)
    body = open(os.path.join(d, "dmrg.conf")).read()
    body = body.replace("orbitals FCIDUMP", "orbitals %s" % os.path.join(d, "FCIDUMP"))
    conf = tmp_path / "dmrg.conf"
    conf.write_text(body + "%s\nprefix %s\n" % (keyword, tmp_path))
    return str(conf)


def check_golden_onepdm(name, pdms, get, tmp_path):
    """The reference's own 1-RDM tables (test_onepdm.py: sum of squared
    differences within 1e-7; test_transitiononepdm.py: the same, up to an
    overall sign of the transition matrix) against `get(bra, ket)` and the
    files the run wrote."""
    norb = None
    for p in pdms:
        gr = read_spatial_onepdm(os.path.join(GOLDEN, name, p["file"]))
        norb = gr.shape[0]
        g = get(p["bra"], p["ket"], norb)
        d = min(np.sum((g - gr) ** 2), np.sum((g + gr) ** 2) if p["bra"] != p["ket"] else np.inf)
        assert d <= p["sumsq"], (name, p["file"], d)
        gt = read_spatial_onepdm(tmp_path / ("spatial_onepdm.%d.%d.txt" % (p["bra"], p["ket"])))
        assert np.max(np.abs(gt - g)) <= 1e-13 * np.max(np.abs(g))


@pytest.mark.parametrize("name,pdms", golden_onepdm_cases(), ids=lambda x: x if isinstance(x, str) else "")
def test_onepdm_matches_reference_tables(oracle, tmp_path, name, pdms):
    conf = onepdm_golden_conf(tmp_path, name, "tran_onepdm")
    oracle.run(conf)
    check_golden_onepdm(name, pdms, lambda a, b, n: oracle.transition_onepdm(a, b, n), tmp_path)
    # bra == ket is the root's density matrix
    for r in range(2):
        assert np.array_equal(oracle.transition_onepdm(r, r, 8 if name == "hubbard" else 7),
                              oracle.onepdm(r, 8 if name == "hubbard" else 7))
