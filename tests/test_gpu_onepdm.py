"""The one-particle density matrix sweep on the GPU (the onepdm keyword,
bgpu_onepdm; modules/onepdm/onepdm.C) against the determinant FCI and the
oracle.

Tolerances written here:
  - the 8-orbital cases (exact at M=200, final solves to 1e-12) against the
    FCI gamma within the oracle's own bounds (1e-6; 2e-6 for the second
    state-averaged Hubbard root), and against the oracle within the same;
  - the truncating 16-orbital M=200 case against the oracle within 1e-5
    elementwise, both started from the unit-vector guess (the two runs'
    sweep energies differ by about 1e-7 Eh, and gamma is first order in the
    wavefunction's difference), with the same trace as the oracle's to
    1e-5 (the trace is not 16 here: each element comes from the step of
    the sweep that holds its operators, and the steps' truncated
    wavefunctions differ by the discarded weight, up to 1e-2);
  - the same case in split precision (bf16x3tc with defect correction)
    against the FP64 GPU gamma within 1e-5;
  - the reference's own 1-RDM tables (Hubbard roots 0 and 1, C2v water
    roots 0 and 1 and <1|E_kl|0>) within its measure, a sum of squared
    differences at most 1e-7, and the transition matrices within 1e-4 of
    the oracle's (these schedules end with Davidson tolerance 1e-8 on the
    squared residual, and the GPU solves start from transformed guesses:
    observed 2.4e-5; 1e-4 is about the tables' own elementwise measure);
  - the 8-orbital cases' transition matrices (two state-averaged roots)
    against the FCI ones up to one overall sign, within the same bounds as
    the roots' own matrices."""
import numpy as np
import pytest

from conftest import conf
from test_oracle_fci import write_fcidump
from test_oracle_onepdm import (CASES, check_golden_onepdm, fci_onepdm, golden_onepdm_cases, onepdm_conf,
                                onepdm_golden_conf, read_spatial_onepdm)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,spin,reorder,tol", CASES)
def test_onepdm_matches_fci_and_oracle(gpu_ctx, oracle, tmp_path, name, spin, reorder, tol):
    c = onepdm_conf(tmp_path, name, spin, reorder)
    t, v, ecore = write_fcidump(oracle, c, str(tmp_path / "FCIDUMP"), input_order=True)
    eo, _ = oracle.run(c)
    go = [oracle.onepdm(r, 8) for r in range(len(eo))]
    e, _ = gpu_ctx.run_dmrg(c)
    for r in range(len(e)):
        g = gpu_ctx.onepdm(r, 8)
        gf = fci_onepdm(t, v, ecore, 8, e[r])
        assert np.max(np.abs(g - gf)) <= tol, (r, np.max(np.abs(g - gf)))
        assert np.max(np.abs(g - go[r])) <= tol, (r, np.max(np.abs(g - go[r])))
        assert abs(np.trace(g) - 8) <= tol
        gt = read_spatial_onepdm(tmp_path / ("spatial_onepdm.%d.%d.txt" % (r, r)))
        assert np.max(np.abs(gt - g)) <= 1e-13 * np.max(np.abs(g))
    if len(e) > 1:
        gf = fci_onepdm(t, v, ecore, 8, e[1], ket_energy=e[0])
        for a, b, ref in ((1, 0, gf), (0, 1, gf.T)):
            g = gpu_ctx.transition_onepdm(a, b, 8)
            d = min(np.max(np.abs(g - ref)), np.max(np.abs(g + ref)))
            assert d <= tol, (a, b, d)


@pytest.fixture
def unit_guess(gpu_ctx):
    gpu_ctx.set_guess(False)
    yield gpu_ctx
    gpu_ctx.set_guess(True)
    gpu_ctx.set_precision("fp64")


def test_onepdm_truncating_case(unit_guess, oracle, tmp_path):
    ctx = unit_guess
    c = tmp_path / "dmrg.conf"
    c.write_text(open(conf("syn16_m200")).read() + "onepdm\n")
    eo, _ = oracle.run(str(c))
    go = oracle.onepdm(0, 16)
    ctx.run_dmrg(str(c))
    g64 = ctx.onepdm(0, 16)
    assert np.max(np.abs(g64 - go)) <= 1e-5, np.max(np.abs(g64 - go))
    assert abs(np.trace(g64) - np.trace(go)) <= 1e-5
    ctx.set_precision("bf16x3tc")
    ctx.run_dmrg(str(c))
    gs = ctx.onepdm(0, 16)
    assert np.max(np.abs(gs - g64)) <= 1e-5, np.max(np.abs(gs - g64))


def test_onepdm_needs_the_keyword(gpu_ctx):
    import block_gb300

    gpu_ctx.run_dmrg(conf("syn8"))
    with pytest.raises(block_gb300.BgpuError):
        gpu_ctx.onepdm(0, 8)


@pytest.mark.parametrize("name,pdms", golden_onepdm_cases(), ids=lambda x: x if isinstance(x, str) else "")
def test_onepdm_matches_reference_tables(gpu_ctx, oracle, tmp_path, name, pdms):
    c = onepdm_golden_conf(tmp_path, name, "tran_onepdm")
    oracle.run(c)
    n = 8 if name == "hubbard" else 7
    go = {(a, b): oracle.transition_onepdm(a, b, n) for a in range(2) for b in range(2)}
    gpu_ctx.run_dmrg(c)
    check_golden_onepdm(name, pdms, lambda a, b, m: gpu_ctx.transition_onepdm(a, b, m), tmp_path)
    for (a, b), g in go.items():
        gg = gpu_ctx.transition_onepdm(a, b, n)
        d = min(np.max(np.abs(gg - g)), np.max(np.abs(gg + g)) if a != b else np.inf)
        assert d <= 1e-4, (a, b, d)
