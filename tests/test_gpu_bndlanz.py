"""Lanczos bound states with the GPU's FP64 H psi (mw3_hphi, host arrays, as
bndgrid's Hmatrix calls difs) against the same recursion with the oracle's
H psi: recursion coefficients, converged eigenvalues and CG eigenvectors."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["tiny_j0", "tiny_j3"])
def test_gpu_lanczos_matches_oracle(runs, case):
    from madwave3_gb300 import Propagator, bndlanz
    from madwave3_gb300.host.constants import ev_to_zot
    from oracle.mw3ref import Oracle

    run = runs[case]
    p = Propagator(run, "fp64")
    o = Oracle(run)
    v1 = bndlanz.initial_vector(run, run.vmintot + ev_to_zot(1.0))
    etg, ag, bg = bndlanz.lanczos_eigenvalues(p.hphi, v1, nkrymax=300, ntimes=150)
    eto, ao, bo = bndlanz.lanczos_eigenvalues(o.hphi, v1, nkrymax=300, ntimes=150)
    # without reorthogonalisation rounding differences grow along the recursion;
    # the first 40 coefficients agree to near FP64 rounding
    assert np.max(np.abs(ag[:40] - ao[:40])) < 1e-10 * np.max(np.abs(ao[:40]))
    assert np.max(np.abs(bg[:40] - bo[:40])) < 1e-10 * np.max(np.abs(bo[:40]))
    assert np.max(np.abs(etg[:3] - eto[:3])) < 1e-10
    e0 = float(eto[0])
    crit = ev_to_zot(1e-6)
    vg, emg, _, okg = bndlanz.cg_eigenvector(p.hphi, v1, e0, 3000, crit)
    vo, emo, _, oko = bndlanz.cg_eigenvector(o.hphi, v1, e0, 3000, crit)
    assert okg and oko
    assert abs(np.dot(vg, vo)) > 0.99999
    p.close()
