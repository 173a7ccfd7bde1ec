"""Per-iteration Cvj / Cvjprod on the device (the reference's Cvj.NNNN and
Cvjprod.NNNN records, SRC/main_madwave3.f:310-321, 354-364): the history ring
against the oracle's Cvj after each iteration, across CUDA-graph replays and
the ring's wrap, and the files written from it."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 5e-4)])
def test_cvj_history_against_the_oracle(runs, precision, tol, tmp_path):
    from madwave3_gb300 import Propagator, contfiles
    from oracle.mw3ref import Oracle

    run = runs["tiny_j3"]
    ref = Oracle(run)
    ref.start(run.psi0)
    per_it = []
    for _ in range(70):
        ref.run_iters(1)
        per_it.append(ref.s2()[1].copy())
    per_it = np.array(per_it)                   # iterations 2..71
    p = Propagator(run, precision)
    p.cvj_history(48)                           # fewer slots than iterations: the ring wraps
    p.start()
    p.run(70)                                   # eager iterations and a 32-iteration graph block
    its, cvj, cp = p.download_cvj_history(48)
    assert cp is None
    assert list(its) == list(range(71 - 47, 72))
    assert cvj.shape == (48,) + per_it.shape[1:]
    assert rel(cvj, per_it[-48:]) < tol
    path = str(tmp_path / "Cvj.0001")
    contfiles.write_cvj_file(path, its, cvj)
    its2, cvj2 = contfiles.read_cvj_file(path, cvj.shape[1:])
    assert np.array_equal(its2, its) and np.array_equal(cvj2, cvj)
    p.close()


def test_cvjprod_history(runs):
    """With a product projection, Cvjprod of every iteration: the last record
    is the library's last Cvjprod, and the records match a run that reads
    Cvjprod after each single iteration."""
    from conftest import synthetic_product_tables
    from madwave3_gb300 import Propagator

    run = runs["tiny_j3"]
    pp = synthetic_product_tables(run)
    a = Propagator(run, "fp64")
    a.set_product_projection(pp)
    a.cvj_history(40)
    a.start()
    a.run(40)
    its, cvj, cp = a.download_cvj_history(40)
    assert cp.shape == (40,) + pp.shape
    assert np.array_equal(cp[-1], a.product()[1])
    b = Propagator(run, "fp64")
    b.set_product_projection(pp)
    b.start()
    seq = []
    for _ in range(40):
        b.run(1)
        seq.append(b.product()[1].copy())
    assert rel(cp, np.array(seq)) < 1e-13
    a.close()
    b.close()
