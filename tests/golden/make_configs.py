"""Writes the dmrg.conf inputs of the benchmark configurations.

hubbard12: open 12-site Hubbard chain, t=1, U=4, half filling (FCIDUMP
written here).  syn24 / syn30 / syn30_d2h / syn40 (and syn30_sweep1, syn30
for one sweep; syn30_m1000, syn30 at M=1000, the profiling size of the
bench's kernels; syn40_m1000, syn40 at M=1000): seeded synthetic
Cholesky Hamiltonians generated inside the library from the `orbitals
synthetic:<norb>:<nelec>:<nchol>:<seed>:<d2h>` spec; syn8 / syn8_d2h are
small members of the same family used for FCI cross-checks; syn20_d2h (20
orbitals, D2h irreps, M=300) is a small batching case of many uneven
sectors.  syn16_m200
(16 orbitals, M=200, 4 sweeps) and syn24_m250_s2 (two sweeps of the
24-orbital system at M=250) truncate heavily: the split-precision sweeps are
compared with the FP64 ones sweep by sweep on them, with Davidson converged
to 1e-12 so that the comparison is not limited by the FP64 run's own solver
tolerance.  syn16_noise
runs syn16_m200 with perturbative noise in its first two sweeps and random
noise in the first.
"""
import os

HERE = os.path.dirname(os.path.abspath(__file__))


def hubbard_fcidump(path, n=12, t=1.0, u=4.0):
    with open(path, "w") as f:
        f.write(" &FCI NORB=%d,NELEC=%d,MS2=0,\n  ORBSYM=%s\n  ISYM=1\n &END\n" % (n, n, ",".join(["1"] * n)))
        for i in range(1, n + 1):
            f.write("%20.12f %4d %4d %4d %4d\n" % (u, i, i, i, i))
        for i in range(1, n):
            f.write("%20.12f %4d %4d %4d %4d\n" % (-t, i + 1, i, 0, 0))
        f.write("%20.12f %4d %4d %4d %4d\n" % (0.0, 0, 0, 0, 0))


CONFS = {
    "hubbard12": ("FCIDUMP", "nelec 12\nspin 0\nschedule\n0 50 1e-8 0\n2 100 1e-8 0\nend\nmaxiter 4\nsweep_tol 1e-12\nnoreorder\n"),
    "syn8": ("synthetic:8:8:16:8:0", "nelec 8\nspin 0\nschedule\n0 200 1e-12 0\nend\nmaxiter 6\nsweep_tol 1e-12\nnoreorder\n"),
    "syn8_d2h": ("synthetic:8:8:16:8:1", "nelec 8\nspin 0\nschedule\n0 200 1e-12 0\nend\nmaxiter 6\nsweep_tol 1e-12\nnoreorder\n"),
    "syn24": ("synthetic:24:24:48:24:0", "nelec 24\nspin 0\nschedule\n0 500 1e-8 0\nend\nmaxiter 6\nsweep_tol 1e-12\nnoreorder\n"),
    "syn24_m250": ("synthetic:24:24:48:24:0", "nelec 24\nspin 0\nschedule\n0 250 1e-8 0\nend\nmaxiter 6\nsweep_tol 1e-12\nnoreorder\n"),
    "syn16_m200": ("synthetic:16:16:32:16:0", "nelec 16\nspin 0\nschedule\n0 200 1e-12 0\nend\nmaxiter 4\nsweep_tol 1e-12\nnoreorder\n"),
    "syn16_noise": ("synthetic:16:16:32:16:0", "nelec 16\nspin 0\nschedule\n0 200 1e-12 1e-4\n2 200 1e-12 0\nend\n"
                    "maxiter 4\nsweep_tol 1e-12\nnoreorder\ntwodot_noise 1e-3 0.5\n"),
    "syn24_m250_s2": ("synthetic:24:24:48:24:0", "nelec 24\nspin 0\nschedule\n0 250 1e-12 0\nend\nmaxiter 2\n"
                      "sweep_tol 1e-12\nnoreorder\n"),
    "syn30": ("synthetic:30:30:60:30:0", "nelec 30\nspin 0\nschedule\n0 2000 1e-8 0\nend\nmaxiter 4\nsweep_tol 1e-12\nnoreorder\n"),
    "syn30_sweep1": ("synthetic:30:30:60:30:0", "nelec 30\nspin 0\nschedule\n0 2000 1e-8 0\nend\nmaxiter 1\nsweep_tol 1e-12\nnoreorder\n"),
    "syn30_m1000": ("synthetic:30:30:60:30:0", "nelec 30\nspin 0\nschedule\n0 1000 1e-8 0\nend\nmaxiter 4\nsweep_tol 1e-12\nnoreorder\n"),
    "syn30_d2h": ("synthetic:30:30:60:30:1", "nelec 30\nspin 0\nschedule\n0 1500 1e-8 0\nend\nmaxiter 4\nsweep_tol 1e-12\nnoreorder\n"),
    "syn20_d2h": ("synthetic:20:20:40:20:1", "nelec 20\nspin 0\nschedule\n0 300 1e-8 0\nend\nmaxiter 2\nsweep_tol 1e-12\nnoreorder\n"),
    "syn40_m1000": ("synthetic:40:40:80:40:0", "nelec 40\nspin 0\nnroots 3\nweights 0.333333333333 0.333333333333 0.333333333334\nschedule\n0 1000 1e-8 0\nend\nmaxiter 2\nsweep_tol 1e-12\nnoreorder\n"),
    "syn40": ("synthetic:40:40:80:40:0", "nelec 40\nspin 0\nnroots 3\nweights 0.333333333333 0.333333333333 0.333333333334\nschedule\n0 4000 1e-8 0\nend\nmaxiter 2\nsweep_tol 1e-12\nnoreorder\n"),
}


def main():
    for name, (orb, body) in CONFS.items():
        d = os.path.join(HERE, name)
        os.makedirs(d, exist_ok=True)
        if orb == "FCIDUMP":
            hubbard_fcidump(os.path.join(d, "FCIDUMP"))
        with open(os.path.join(d, "dmrg.conf"), "w") as f:
            f.write(body + "orbitals %s\n" % orb)


if __name__ == "__main__":
    main()
