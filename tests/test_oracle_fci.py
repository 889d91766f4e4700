"""The oracle's spin-adapted DMRG on small members of the synthetic
Hamiltonian family (C1 and D2h) against an independent determinant FCI in
numpy: the DMRG energies of the S=0, 1, 2 targets are eigenvalues of the FCI
Hamiltonian, and their minimum is the FCI ground state (1e-8 Eh)."""
import itertools
import os
import subprocess

import numpy as np
import pytest
import scipy.sparse as sp
import scipy.sparse.linalg as sla

from conftest import GOLDEN


def read_fcidump(path):
    with open(path) as f:
        txt = f.read()
    head, body = txt.upper().split("&END")
    norb = int(head.split("NORB=")[1].split(",")[0])
    t = np.zeros((norb, norb))
    v = np.zeros((norb,) * 4)
    ecore = 0.0
    for line in body.strip().splitlines():
        x, i, j, k, l = line.split()
        x = float(x)
        i, j, k, l = int(i), int(j), int(k), int(l)
        if i == j == k == l == 0:
            ecore = x
        elif k == 0 and l == 0:
            t[i - 1, j - 1] = t[j - 1, i - 1] = x
        else:
            i, j, k, l = i - 1, j - 1, k - 1, l - 1
            for a, b, c, d in ((i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k)):
                v[a, b, c, d] = v[c, d, a, b] = x
    return t, v, ecore


def fci_operators(t, v, ecore, nelec):
    """The determinant-space Hamiltonian (M_S = 0) and the spin-summed
    excitation operators E_pq = a+_pa a_qa + a+_pb a_qb as sparse matrices."""
    n = t.shape[0]
    na = nelec // 2
    strs = [sum(1 << o for o in c) for c in itertools.combinations(range(n), na)]
    idx = {s: i for i, s in enumerate(strs)}
    ns = len(strs)

    def excit(p, q):
        rows, cols, vals = [], [], []
        for s in strs:
            if not (s >> q) & 1:
                continue
            s1 = s & ~(1 << q)
            if (s1 >> p) & 1:
                continue
            sign = (-1) ** bin(s1 & ((1 << q) - 1)).count("1")
            sign *= (-1) ** bin(s1 & ((1 << p) - 1)).count("1")
            s2 = s1 | (1 << p)
            rows.append(idx[s2])
            cols.append(idx[s])
            vals.append(sign)
        return sp.csr_matrix((vals, (rows, cols)), shape=(ns, ns))

    I = sp.identity(ns, format="csr")
    # alpha strings are the slower index; beta operators pass the alpha string
    # with a sign that cancels in the number-conserving E_pq
    E = {}
    for p in range(n):
        for q in range(n):
            e = excit(p, q)
            E[p, q] = sp.kron(e, I, format="csr") + sp.kron(I, e, format="csr")
    H = ecore * sp.identity(ns * ns, format="csr")
    for p in range(n):
        for q in range(n):
            if t[p, q] != 0:
                H = H + t[p, q] * E[p, q]
    for p in range(n):
        for q in range(n):
            W = None
            for r in range(n):
                for s in range(n):
                    if v[p, q, r, s] != 0:
                        W = v[p, q, r, s] * E[r, s] if W is None else W + v[p, q, r, s] * E[r, s]
            if W is not None:
                H = H + 0.5 * (E[p, q] @ W)
    for p in range(n):
        for s in range(n):
            c = sum(v[p, q, q, s] for q in range(n))
            if c != 0:
                H = H - 0.5 * c * E[p, s]
    return H, E


def fci_energies(t, v, ecore, nelec, nroots=12):
    H, _ = fci_operators(t, v, ecore, nelec)
    w = sla.eigsh(H, k=nroots, which="SA", tol=1e-12)[0]
    return np.sort(w)


def write_fcidump(oracle, conf, path, input_order=False):
    """The generated integrals of a configuration, through the oracle CLI's
    FCIDUMP writer: in the sweep's orbital order, or in the input order."""
    exe = os.path.join(os.path.dirname(oracle.LIB), "dmrg_oracle")
    args = [exe, conf, "--write-fcidump", path] + (["--noreorder"] if input_order else [])
    subprocess.run(args, check=True, capture_output=True)
    return read_fcidump(path)


@pytest.mark.parametrize("name", ["syn8", "syn8_d2h"])
def test_dmrg_spin_sectors_are_fci_eigenvalues(oracle, name, tmp_path):
    base = os.path.join(GOLDEN, name, "dmrg.conf")
    with open(base) as f:
        body = f.read()
    t, v, ecore = write_fcidump(oracle, base, str(tmp_path / "FCIDUMP"))
    w = fci_energies(t, v, ecore, 8, nroots=120)
    es = []
    for spin in (0, 2, 4):
        conf = tmp_path / ("s%d.conf" % spin)
        conf.write_text(body.replace("spin 0", "spin %d" % spin))
        e, _ = oracle.run(str(conf))
        assert np.min(np.abs(w - e[0])) <= 1e-8, (spin, e[0], w[:6])
        es.append(e[0])
    assert abs(min(es) - w[0]) <= 1e-8, (es, w[0])
