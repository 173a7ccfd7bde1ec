"""prodpaq / prodcvj on the GPU (mw3_set_product_projection) against the
oracle's, on seeded tables: FP64 within 1e-10, the mixed path within the
accuracy of its state, graph replay included (70 iterations)."""
import numpy as np
import pytest

from conftest import synthetic_product_tables

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 5e-4)])
@pytest.mark.parametrize("case", ["tiny_j3", "tiny_e2"])
def test_gpu_product_projection(runs, case, precision, tol):
    from madwave3_gb300 import Propagator
    from oracle.mw3ref import Oracle

    run = runs[case]
    pp = synthetic_product_tables(run)
    o = Oracle(run)
    o.set_product(pp)
    o.start(run.psi0)
    o.run_iters(70)
    zo, co = o.product()
    p = Propagator(run, precision)
    p.set_product_projection(pp)
    p.start()
    p.run(70)
    zg, cg = p.product()
    assert np.max(np.abs(cg - co)) <= tol * np.max(np.abs(co))
    assert np.max(np.abs(zg - zo)) <= tol * np.max(np.abs(zo))
    assert np.all(zg[co == 0] == 0)
    p.close()


def test_product_projection_must_precede_the_device_tables(runs):
    from madwave3_gb300 import Mw3Error, Propagator

    run = runs["tiny_j3"]
    p = Propagator(run, "fp64")
    p.hphi(np.ones(run.ntot))
    with pytest.raises(Mw3Error):
        p.set_product_projection(synthetic_product_tables(run))
    p.close()


def test_gpu_product_chain_from_host_setup(runs):
    """The projection with ini_transcoor's tables built on the host from the
    synthetic product states (FP64 path against the oracle)."""
    from madwave3_gb300 import Propagator
    from madwave3_gb300.host import generator, transcoor
    from oracle.mw3ref import Oracle

    run = runs["tiny_j3"]
    fd, ed, nob = generator.product_states(run, 30, 0, 4, 0, 2, **generator.CASES["tiny_j3"])
    pp = transcoor.ini_transcoor(run, 1.8, 3, 30, 1, run.inp.nangu, 0, 2, 0, 4, 0, 2, nob, fd)
    o = Oracle(run)
    o.set_product(pp)
    o.start(run.psi0)
    o.run_iters(40)
    zo, co = o.product()
    p = Propagator(run, "fp64")
    p.set_product_projection(pp)
    p.start()
    p.run(40)
    zg, cg = p.product()
    p.close()
    assert np.abs(zo).max() > 0
    assert np.max(np.abs(zg - zo)) <= 1e-10 * np.max(np.abs(zo))
    assert np.max(np.abs(cg - co)) <= 1e-10 * np.max(np.abs(co))
