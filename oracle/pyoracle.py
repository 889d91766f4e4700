"""TEST INFRASTRUCTURE ONLY: ctypes access to the CPU oracle (liboracle.so).

Used by tests/ and by bench.py's CPU-baseline leg; never by block_gb300.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "_build", "liboracle.so")
EXE = os.path.join(HERE, "_build", "dmrg_oracle")
_lib = None


def build():
    subprocess.run(["make", "-s", "-C", HERE, "-j", str(min(16, os.cpu_count() or 4))], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = ctypes.CDLL(LIB)
        P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        DP = ctypes.POINTER(ctypes.c_double)
        L.oracle_run.restype = I
        L.oracle_run.argtypes = [ctypes.c_char_p, I, I, DP, I, DP]
        L.oracle_snapshot.restype = P
        L.oracle_snapshot.argtypes = [ctypes.c_char_p, I, I, I]
        L.oracle_prepare.restype = P
        L.oracle_prepare.argtypes = [ctypes.c_char_p, I, I, I, I]
        L.oracle_snapshot_free.argtypes = [P]
        L.oracle_snapshot_sizes.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
        L.oracle_snapshot_block.argtypes = [P, I, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I), DP]
        L.oracle_snapshot_data.argtypes = [P, DP, ctypes.POINTER(I), DP, DP, DP, ctypes.POINTER(I), DP]
        L.oracle_snapshot_group.restype = ctypes.c_char_p
        L.oracle_snapshot_group.argtypes = [P]
        L.oracle_time_sigma.restype = D
        L.oracle_time_sigma.argtypes = [ctypes.c_char_p, I, I, I, I]
        _lib = L
    return _lib


# ---------------------------------------------------------------- BLAS
# The reference links a tuned BLAS for its DGEMMs (CMakeLists.txt:31-47);
# the oracle can route its DGEMM through the OpenBLAS that SciPy bundles, so
# that the CPU baseline is not held back by the built-in loop.  A library is
# used only after a child process has run the oracle with it and matched the
# built-in products, so a mismatched library cannot take down the caller.
_blas = None  # (path or None, description)


def blas_candidates():
    import glob

    out = []
    try:
        import scipy

        base = os.path.dirname(os.path.dirname(scipy.__file__))
        out += sorted(glob.glob(os.path.join(base, "scipy.libs", "libscipy_openblas*.so*")))
    except ImportError:
        pass
    try:
        import scipy_openblas32

        out += sorted(glob.glob(os.path.join(os.path.dirname(scipy_openblas32.__file__), "lib", "libscipy_openblas*.so*")))
    except ImportError:
        pass
    return [p for p in out if "openblas64" not in os.path.basename(p)]  # 64-bit-integer builds take other symbols


def _blas_selftest(path):
    """Child-process check: sigma of a small superblock with the BLAS equals
    the built-in loop's to 1e-12 (relative)."""
    L = lib()
    L.oracle_use_blas.restype = ctypes.c_int
    L.oracle_use_blas.argtypes = [ctypes.c_char_p]
    conf = os.path.join(os.path.dirname(HERE), "tests", "golden", "hubbard", "dmrg.conf")
    ref = snapshot(conf, 1, 3)
    if L.oracle_use_blas(path.encode()) != 0:
        return 1
    got = snapshot(conf, 1, 3)
    err = np.linalg.norm(got["sigma"] - ref["sigma"]) / np.linalg.norm(ref["sigma"])
    return 0 if err <= 1e-12 else 2


def enable_blas():
    """Use the first candidate BLAS that passes the child-process check;
    returns a description of the DGEMM in use."""
    global _blas
    if _blas is not None:
        return _blas[1]
    import sys

    L = lib()
    L.oracle_use_blas.restype = ctypes.c_int
    L.oracle_use_blas.argtypes = [ctypes.c_char_p]
    for path in blas_candidates():
        code = "import sys; sys.path.insert(0, %r); import pyoracle; sys.exit(pyoracle._blas_selftest(%r))" % (HERE, path)
        try:
            rc = subprocess.run([sys.executable, "-c", code], capture_output=True, timeout=300).returncode
        except (OSError, subprocess.TimeoutExpired):
            rc = -1
        if rc == 0 and L.oracle_use_blas(path.encode()) == 0:
            _blas = (path, "OpenBLAS bundled with SciPy (%s), one thread per operator-pair worker" % os.path.basename(path))
            return _blas[1]
    _blas = (None, "built-in cache-blocked loop")
    return _blas[1]


def disable_blas():
    """Back to the built-in DGEMM loop."""
    global _blas
    L = lib()
    L.oracle_use_blas.restype = ctypes.c_int
    L.oracle_use_blas.argtypes = [ctypes.c_char_p]
    L.oracle_use_blas(None)
    _blas = None


def run(conf, threads=0, verbose=0, max_roots=32, guess=False):
    """A whole run of dmrg.conf on the oracle; guess=True starts every
    Davidson solve it can from the transformed previous wavefunction."""
    L = lib()
    L.oracle_set_guess.restype = ctypes.c_int
    L.oracle_set_guess.argtypes = [ctypes.c_int]
    L.oracle_set_guess(int(bool(guess)))
    e = np.zeros(max_roots)
    st = np.zeros(12)
    rc = L.oracle_run(conf.encode(), threads, verbose, e.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), max_roots,
                      st.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
    if rc != 0:
        raise RuntimeError("oracle run failed for " + conf)
    n = int(st[7])
    L.oracle_sweep_energies.restype = ctypes.c_int
    L.oracle_sweep_energies.argtypes = [ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    sw = np.zeros(256)
    ns = L.oracle_sweep_energies(sw.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), len(sw))
    return e[:n].copy(), dict(sweeps=int(st[0]), sigma_calls=int(st[1]), sigma_seconds=st[2], seconds=st[4],
                              discarded=st[5], last_sweep_energy=st[6], sweep_energies=sw[:min(ns, 256)].copy(),
                              spill_fetches=int(st[8]), spill_bytes_up=st[9], spill_bytes_down=st[10],
                              peak_block_bytes=st[11])


def su2(kind, *args):
    """Spin-coupling coefficient of the shared host code (2j arguments):
    kind "clebsch" (j1 m1 j2 m2 j3 m3), "six_j", "nine_j", "ninej" (the
    normalised 9j of the coupling tables) or "transpose_scaling" (l r k)."""
    kinds = {"clebsch": 0, "six_j": 1, "nine_j": 2, "ninej": 3, "transpose_scaling": 4}
    L = lib()
    L.oracle_su2.restype = ctypes.c_int
    L.oracle_su2.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)]
    a = (ctypes.c_int * 9)(*args)
    out = ctypes.c_double()
    rc = L.oracle_su2(kinds[kind], a, ctypes.byref(out))
    if rc:
        raise ValueError("%s%r refused (%d)" % (kind, args, rc))
    return out.value


def _ptr(a, t):
    return a.ctypes.data_as(ctypes.POINTER(t))


def _unpack(L, h):
    if not h:
        raise RuntimeError("oracle snapshot failed")
    sz = np.zeros(11, dtype=np.int64)
    L.oracle_snapshot_sizes(h, sz.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)))
    snap = {}
    for which, (nq, nops, na) in ((0, sz[0:3]), (1, sz[3:6])):
        q = np.zeros(3 * nq, dtype=np.int32)
        s = np.zeros(nq, dtype=np.int32)
        k = np.zeros(4 * nops, dtype=np.int32)
        a = np.zeros(na, dtype=np.float64)
        L.oracle_snapshot_block(h, which, _ptr(q, ctypes.c_int), _ptr(s, ctypes.c_int), _ptr(k, ctypes.c_int),
                                _ptr(a, ctypes.c_double))
        snap["L" if which == 0 else "R"] = dict(quanta=q.reshape(-1, 3), states=s, keys=k.reshape(-1, 4), arena=a,
                                                is_dot=int(sz[9 + which]))
    nt, n, norb = int(sz[6]), int(sz[7]), int(sz[8])
    coef = np.zeros(nt)
    ops = np.zeros(4 * nt, dtype=np.int32)
    psi = np.zeros(n)
    sig = np.zeros(n)
    diag = np.zeros(n)
    orbsym = np.zeros(norb, dtype=np.int32)
    misc = np.zeros(9)
    L.oracle_snapshot_data(h, _ptr(coef, ctypes.c_double), _ptr(ops, ctypes.c_int), _ptr(psi, ctypes.c_double),
                           _ptr(sig, ctypes.c_double), _ptr(diag, ctypes.c_double), _ptr(orbsym, ctypes.c_int),
                           _ptr(misc, ctypes.c_double))
    snap.update(coef=coef, ops=ops.reshape(-1, 4), psi=psi, sigma=sig, diag=diag, orbsym=orbsym,
                target=misc[0:3].astype(np.int32), ecore=misc[3], energy=misc[4], sigma_seconds=misc[5],
                threads=int(misc[6]), flops=misc[7], sigma_seconds_1t=misc[8],
                group=L.oracle_snapshot_group(h).decode())
    L.oracle_snapshot_free(h)
    return snap


def snapshot(conf, sweep, pos, threads=0):
    """Superblock of step (sweep, pos) of an oracle run, with psi = root 0."""
    L = lib()
    return _unpack(L, L.oracle_snapshot(conf.encode(), sweep, pos, threads))


def prepare(conf, partition, threads=0, reps=1, time_single=False):
    """Superblock built from seeded warm-up blocks (see bgpu_prepare_superblock);
    the oracle sigma is timed over `reps` products (seconds per product), and
    with time_single also once on one thread (sigma_seconds_1t)."""
    L = lib()
    return _unpack(L, L.oracle_prepare(conf.encode(), partition, threads, reps, int(bool(time_single))))


def time_sigma(conf, sweep, pos, threads=0, reps=3):
    return lib().oracle_time_sigma(conf.encode(), sweep, pos, threads, reps)


def block_case(conf, partition, threads=0, noise=0.0, random_noise=0.0, seed=0):
    """Element-wise parity case at `partition` of a configuration's warm-up
    chain (see oracle_block_case): system, dot, enlarged and renormalised
    blocks (quanta, states, keys, sites, arenas), the environment block's
    state space, a random wavefunction, its left density matrix (with the
    given perturbative / random noise and seed) with eigenvalues and
    eigenvectors, and the kept rotation."""
    L = lib()
    L.oracle_block_case.restype = ctypes.c_void_p
    L.oracle_block_case.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_double,
                                    ctypes.c_ulonglong]
    L.oracle_case_len.restype = ctypes.c_int64
    L.oracle_case_len.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int]
    L.oracle_case_get.argtypes = [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_int, ctypes.c_void_p]
    L.oracle_case_free.argtypes = [ctypes.c_void_p]
    L.oracle_case_group.restype = ctypes.c_char_p
    L.oracle_case_group.argtypes = [ctypes.c_void_p]
    h = L.oracle_block_case(conf.encode(), partition, threads, float(noise), float(random_noise), int(seed))
    if not h:
        raise RuntimeError("oracle block case failed")
    out = {"group": L.oracle_case_group(h).decode()}
    names_i = ["orbsym", "filter", "target", "kept"]
    names_d = ["psi", "rho", "vecs", "eig", "rot"]
    for b in ("sys", "dot", "big", "env", "small"):
        names_i += [b + "_quanta", b + "_states", b + "_keys", b + "_sites"]
        names_d += [b + "_arena"]
    for kind, names, dt in ((0, names_i, np.int32), (1, names_d, np.float64)):
        for nm in names:
            n = L.oracle_case_len(h, nm.encode(), kind)
            if n < 0:
                continue
            a = np.zeros(n, dtype=dt)
            if n:
                L.oracle_case_get(h, nm.encode(), kind, a.ctypes.data)
            out[nm] = a
    L.oracle_case_free(h)
    for b in ("sys", "dot", "big", "env", "small"):
        out[b + "_quanta"] = out[b + "_quanta"].reshape(-1, 3)
        out[b + "_keys"] = out[b + "_keys"].reshape(-1, 4)
    return out


def sample_sigma(conf, partition, threads=0, reps=1):
    """Oracle sigma timed on a superblock with the structure of `partition`'s
    warm-up superblock and seeded random operator values (see
    oracle_sample_sigma): dict(flops, psi, arena, seconds, norm, threads)."""
    L = lib()
    L.oracle_sample_sigma.restype = ctypes.c_int
    L.oracle_sample_sigma.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      ctypes.POINTER(ctypes.c_double)]
    out = np.zeros(6)
    if L.oracle_sample_sigma(conf.encode(), partition, threads, reps, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double))):
        raise RuntimeError("oracle sample failed for " + conf)
    return dict(flops=out[0], psi=int(out[1]), arena=int(out[2]), seconds=out[3], norm=out[4], threads=int(out[5]))


def onepdm(root, norb):
    """One-particle density matrix of a root from the last run() of a
    configuration with the onepdm keyword."""
    L = lib()
    L.oracle_onepdm.restype = ctypes.c_int
    L.oracle_onepdm.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    g = np.zeros((norb, norb))
    if L.oracle_onepdm(root, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), norb):
        raise RuntimeError("no one-particle density matrix of root %d" % root)
    return g


def transition_onepdm(bra, ket, norb):
    """<bra|E_ij|ket> between two roots of the last run() of a configuration
    with the onepdm (or tran_onepdm) keyword."""
    L = lib()
    L.oracle_transition_onepdm.restype = ctypes.c_int
    L.oracle_transition_onepdm.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int]
    g = np.zeros((norb, norb))
    if L.oracle_transition_onepdm(bra, ket, g.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), norb):
        raise RuntimeError("no transition density matrix of roots %d, %d" % (bra, ket))
    return g
