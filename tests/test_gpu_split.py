"""Split-precision sigma (bf16 slices on the tensor cores, FP32 accumulation)
against the FP64 oracle, and split-precision Davidson / sweeps with the FP64
Rayleigh-quotient refinement against the golden energies.

Tolerances written here: relative sigma error <= 2e-5 for BF16X3 (3 products,
16-bit operands; observed 2-5e-6), <= 5e-5 for FP16X2 (observed 9e-6 to 4e-5)
and <= 5e-6 for BF16X6 (6 products, FP32-level operands);
refined energies within 1e-8 Eh of the dense FP64 eigenvalue on small
superblocks and within the reference's 1e-6 Eh of its golden energies for
full sweeps."""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN, conf
from test_gpu_sigma import SNAPS, load

pytestmark = pytest.mark.gpu

TOL = {"bf16x3": 2e-5, "bf16x6": 5e-6, "bf16x3tc": 2e-5, "fp16x2tc": 5e-5}

with open(os.path.join(GOLDEN, "golden.json")) as f:
    GOLD = json.load(f)


@pytest.fixture
def split_ctx(gpu_ctx):
    yield gpu_ctx
    gpu_ctx.set_precision("fp64")


@pytest.mark.parametrize("prec", ["bf16x3", "bf16x6", "bf16x3tc", "fp16x2tc"])
@pytest.mark.parametrize("name,sweep,pos", SNAPS)
def test_split_sigma_accuracy(split_ctx, oracle, prec, name, sweep, pos):
    snap = oracle.snapshot(conf(name), sweep, pos)
    sb, n = load(split_ctx, snap)
    split_ctx.set_precision(prec)
    x, y = split_ctx.device_alloc(n), split_ctx.device_alloc(n)
    split_ctx.to_device(x, snap["psi"])
    split_ctx.sigma_timed(sb, x, y, 1)
    got = split_ctx.to_host(y, n)
    err = np.linalg.norm(got - snap["sigma"]) / np.linalg.norm(snap["sigma"])
    split_ctx.device_free(x)
    split_ctx.device_free(y)
    assert err <= TOL[prec], (prec, name, err)


@pytest.mark.parametrize("prec", ["bf16x6", "bf16x3tc"])
@pytest.mark.parametrize("name,sweep,pos", SNAPS[:3])
def test_split_davidson_refined_energy(split_ctx, oracle, prec, name, sweep, pos):
    snap = oracle.snapshot(conf(name), sweep, pos)
    sb, n = load(split_ctx, snap)
    e64, _, _ = split_ctx.davidson(sb, n, nroots=1, tol=1e-12)
    split_ctx.set_precision(prec)
    e, _, _ = split_ctx.davidson(sb, n, nroots=1, tol=1e-9)
    assert abs(e[0] - e64[0]) <= 1e-8, (e[0], e64[0])


@pytest.mark.parametrize("prec", ["bf16x6", "bf16x3tc"])
@pytest.mark.parametrize("name", ["hubbard", "c2_d2h"])
def test_split_sweep_golden(split_ctx, prec, name):
    split_ctx.set_precision(prec)
    e, st = split_ctx.run_dmrg(conf(name))
    for got, ref in zip(e, GOLD[name]["energies"]):
        assert abs(got - ref) <= GOLD[name]["tolerance"], (name, got, ref)
