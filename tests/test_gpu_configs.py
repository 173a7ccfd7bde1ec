"""The GPU paths at the workloads' own sizes: the 256 R x 128 r x 60-angle grid
of the J = 0 workload, the J = 6 wave of the J = 0..40 sweep (7 Omega blocks)
and the J = 10 workload with all 11 Omega blocks coupled.

At these sizes the mixed path runs the kernels the bench times: the fused
tcgen05 DST chain with both 128-lane R tiles (npun2 = 256) and the
production nopr1, and the factorised tcgen05 angular contraction with the 60
angles padded to 64.  Bars: FP64 against the oracle 1e-12 on H psi and 1e-10
on the propagation (norms, P(E), the flux and state-resolved accumulators)
after 200 iterations; mixed against FP64 5e-6 on H psi relative to its
largest element (measured 1.5e-6 to 1.6e-6 here: the 3xTF32 products sum
128-term parity halves along R, four times the K of the toy grids, where the
difference is 3e-7)."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def grid_case(tmp_path_factory):
    from madwave3_gb300.host import generator
    d = str(tmp_path_factory.mktemp("cfg") / "j0_256x128x60")
    generator.write_case(d, **generator.CASES["j0_256x128x60"])
    return d


@pytest.fixture(scope="module")
def j0(grid_case):
    from madwave3_gb300.host import setup
    return setup.load(os.path.join(grid_case, "input.dat"))


def _oracle(run):
    from oracle.mw3ref import Oracle
    return Oracle(run, threads=os.cpu_count() or 1)


def test_j0_fp64_against_the_oracle(j0):
    from madwave3_gb300 import Propagator
    prop = Propagator(j0, "fp64")
    ref = _oracle(j0)
    rng = np.random.default_rng(20261203)
    for _ in range(2):
        psi = rng.uniform(-1, 1, j0.ntot)
        assert rel(prop.hphi(psi), ref.hphi(psi)) < 1e-12
    prop.start()
    ref.start(j0.psi0)
    prop.run(200)
    n_ref = ref.run_iters(200)
    assert rel(prop.norms()[1:], n_ref) < 1e-10
    assert rel(prop.totalflux()[0], ref.totalflux()[0]) < 1e-10
    acc = prop.accumulators()
    zcr, zcdr = ref.flux()
    assert rel(acc["zcr"], zcr) < 1e-10 and rel(acc["zcdr"], zcdr) < 1e-10
    zs2, cvj = ref.s2()
    assert rel(acc["zs2"], zs2) < 1e-10 and rel(acc["cvj"], cvj) < 1e-10
    prop.close()


def _mixed_vs_fp64(runs, waves):
    from madwave3_gb300 import Propagator
    pmx = Propagator(runs, "mixed")
    p64 = Propagator(runs, "fp64")
    rng = np.random.default_rng(11)
    for w in waves:
        psi = rng.uniform(-1, 1, runs[w].ntot)
        assert rel(pmx.hphi(psi, w), p64.hphi(psi, w)) < 5e-6
        assert rel(pmx.hphi(runs[w].psi0, w), p64.hphi(runs[w].psi0, w)) < 5e-6
    path = pmx.path()
    assert path["tc_dst"] and path["tc_dst_fused"] and path["tc_angular"], path
    pmx.close()
    p64.close()


def test_j0_mixed_takes_the_tensor_cores_and_tracks_fp64(j0):
    _mixed_vs_fp64([j0], [0])


def test_sweep_waves_mixed_tracks_fp64(grid_case):
    """J = 6 (Omega = 0..6, 7 blocks chained through the Coriolis coupling)
    and J = 1 of the sweep, batched in one context as the bench runs them."""
    from madwave3_gb300.host import generator, setup
    waves = setup.load_sweep(os.path.join(grid_case, "input.dat"), [1, 6], generator.jsweep_inputs)
    assert [w.ncan for w in waves] == [2, 7]
    _mixed_vs_fp64(waves, [0, 1])


@pytest.fixture(scope="module")
def j10(tmp_path_factory):
    from madwave3_gb300.host import generator, setup
    d = str(tmp_path_factory.mktemp("cfg") / "j10_256x128x60")
    generator.write_case(d, **generator.CASES["j10_256x128x60"])
    return setup.load(os.path.join(d, "input.dat"))


def test_j10_all_omega_blocks(j10):
    """J = 10 with Omega = 0..10 (11 blocks): FP64 H psi against the oracle,
    mixed against FP64, and the first 20 iterations' accumulators."""
    from madwave3_gb300 import Propagator
    assert j10.ncan == 11
    prop = Propagator(j10, "fp64")
    ref = _oracle(j10)
    psi = np.random.default_rng(5).uniform(-1, 1, j10.ntot)
    assert rel(prop.hphi(psi), ref.hphi(psi)) < 1e-12
    prop.start()
    ref.start(j10.psi0)
    prop.run(20)
    n_ref = ref.run_iters(20)
    assert rel(prop.norms()[1:], n_ref) < 1e-10
    zs2, cvj = ref.s2()
    acc = prop.accumulators()
    assert rel(acc["zs2"], zs2) < 1e-10 and rel(acc["cvj"], cvj) < 1e-10
    prop.close()
    _mixed_vs_fp64([j10], [0])
