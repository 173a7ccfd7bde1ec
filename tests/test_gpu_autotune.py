"""Path choices and the autotuner (mw3_set_choices, mw3_autotune) on the GPU.

The layout choices (FP32 rectangle [R][r1] or [r1][R], the explicit angular
kernels' column chunk) leave every result bit for bit as it was; the form
choices (radial DST: fused split-FP16 or 3xTF32 chain, three-kernel tensor-core
DST, CUDA-core FP32 DST; factorised or explicit angular terms; FP64 Rader FFT
or folded dense DST) keep the precision bars of the parity tests.
"""
import os

import numpy as np
import pytest

from madwave3_gb300 import Propagator
from oracle.mw3ref import Oracle

pytestmark = pytest.mark.gpu
NIT = 100


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


def propagate(prop, n=NIT):
    prop.start()
    prop.run(n)
    norms = prop.norms()
    km1, k, it = prop.state()
    return norms, k


@pytest.mark.parametrize("case,precision", [("tiny_j3", "fp64"), ("tiny_j0", "mixed")])
def test_layout_autotune_is_bit_identical(runs, case, precision):
    run = runs[case]
    tuned = Propagator(run, precision)
    choice, ms = tuned.autotune(iterations=64, scope="layout")
    assert ms > 0 and choice["dst"] == -1 and choice["angular"] == -1
    plain = Propagator(run, precision)
    n1, k1 = propagate(tuned)
    n0, k0 = propagate(plain)
    assert np.array_equal(n1, n0) and np.array_equal(k1, k0)
    tuned.close()
    plain.close()


FORMS = [(d, a) for d in (0, 1, 2, 3) for a in (0, 1)]


@pytest.mark.parametrize("dst,ang", FORMS)
def test_each_mixed_form(runs, dst, ang):
    run = runs["tiny_j3"]
    p64 = Propagator(run, "fp64")
    pmx = Propagator(run, "mixed")
    pmx.set_choices({"dst": dst, "angular": ang})
    rng = np.random.default_rng(20261204)
    psi = rng.uniform(-1, 1, run.ntot)
    assert rel(pmx.hphi(psi), p64.hphi(psi)) < 1e-6
    pmx.start()
    path = pmx.path()
    assert path["tc_angular"] == (ang == 1)
    assert path["tc_dst_fused"] == (dst in (0, 1))
    if dst in (0, 1):
        assert path["dst_f16"] == (dst == 0)
    assert path["tc_dst"] == (dst in (0, 1, 2))
    p64.close()
    pmx.close()


@pytest.fixture(scope="module")
def r256(tmp_path_factory):
    """A small case with npun2 = 256, where the FP64 DST along R can be a Rader FFT."""
    from madwave3_gb300.host import generator, setup
    d = str(tmp_path_factory.mktemp("r256") / "case")
    generator.write_case(d, npun2=256, npun1=24, nangu=4, jmax=3, nvmax=1, netot=32, npun1min=8,
                         alpha0_bohr=1.2)
    return setup.load(os.path.join(d, "input.dat"))


@pytest.mark.parametrize("dst", [0, 1])
def test_fp64_dst_factorisations(r256, dst):
    prop = Propagator(r256, "fp64")
    prop.set_choices({"dst": dst})
    ref = Oracle(r256)
    psi = np.random.default_rng(3).uniform(-1, 1, r256.ntot)
    assert rel(prop.hphi(psi), ref.hphi(psi)) < 1e-12
    prop.start()
    assert prop.path()["rader"] == (dst == 1)
    prop.close()


def test_form_autotune_keeps_the_mixed_bar(runs):
    run = runs["tiny_j3"]
    tuned = Propagator(run, "mixed")
    choice, ms = tuned.autotune(iterations=64, scope="all")
    assert ms > 0 and set(choice) == set(Propagator.CHOICES)
    p64 = Propagator(run, "fp64")
    tuned.start()
    p64.start()
    tuned.run(NIT)
    p64.run(NIT)
    p, _ = tuned.totalflux()
    q, _ = p64.totalflux()
    assert np.abs(p - q).max() <= 1e-3 * max(1.0, np.abs(q).max())
    tuned.close()
    p64.close()


def test_autotune_after_start_is_refused(runs):
    run = runs["tiny_j0"]
    prop = Propagator(run, "mixed")
    prop.start()
    with pytest.raises(RuntimeError, match="mw3_autotune"):
        prop.autotune(scope="layout")
    with pytest.raises(RuntimeError, match="mw3_set_choices"):
        prop.set_choices({"dst": 3})
    prop.close()
