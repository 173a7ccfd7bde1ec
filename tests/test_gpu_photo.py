"""Photodissociation (iphoto = 1) on the GB300 against the oracle: a J = 1
packet made from a stored J = 0 bound state with a constant transition dipole,
propagated with Smatini_photo's normalisations; check's autocorrelation
<psi0|psi_k>, the norm trace, P(E) and the reactant-channel accumulators."""
import copy
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
NIT = 80


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def photo_case(case_dirs, tmp_path_factory):
    from madwave3_gb300 import bndlanz, photo
    from madwave3_gb300.host import generator, setup
    r0, r1 = setup.load_sweep(os.path.join(case_dirs["tiny_e2"], "input.dat"), [0, 1], generator.jsweep_inputs)
    r1 = copy.copy(r1)
    r1.inp = copy.copy(r1.inp)
    r1.inp.iphoto = 1
    d = str(tmp_path_factory.mktemp("bnd"))
    rng = np.random.default_rng(11)
    vec = rng.standard_normal(r0.ntot)
    bndlanz.write_bnd(d, r0, 0, -0.02, vec / np.linalg.norm(vec))
    dip = photo.dipole_table(r1, lambda r, R, c: (0.3, 0.0, 1.0))
    psi0, pnorm, _, per_om = photo.initial_packet(r1, d, 0, 1, Jtotini=0, iparini=1, dipol=dip)
    assert per_om[1] > 0                       # d_x couples Omega_ini = 0 to Omega = 1
    return r1, psi0


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-10), ("mixed", 1e-4)])
def test_photodissociation_against_the_oracle(photo_case, precision, tol):
    from madwave3_gb300 import Propagator
    from oracle.mw3ref import Oracle
    run, psi0 = photo_case
    ref = Oracle(run)
    ref.start(psi0)
    n_ref, a_ref = ref.run_autocorrelation(NIT)
    p = Propagator(run, precision)
    p.start([psi0])
    p.run(NIT)
    autos = p.autocorrelation()
    assert autos.size == NIT + 1             # slot 0: k = 1, after mw3_start
    assert rel(autos[1:], a_ref) < tol
    assert rel(p.norms()[1:], n_ref) < tol
    assert rel(p.totalflux()[0], ref.totalflux()[0]) < 10 * tol
    zs2, cvj = ref.s2()
    acc = p.accumulators()
    assert rel(acc["zs2"], zs2) < 10 * tol and rel(acc["cvj"], cvj) < 10 * tol
    t, ft = p.tables(), ref.flux_tables()
    assert rel(t["reacfct"], ft["reacfct"]) < 1e-14 and np.all(t["apaqini"] == 0)
    p.close()
