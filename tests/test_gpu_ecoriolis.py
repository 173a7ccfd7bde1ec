"""The electronic Coriolis variant on the GPU (mw3_set_ecoriolis) against the
CPU oracle, through the C-ABI.

tiny_ecor: two coupled states with Lambda = 0 and 1, J = 2, Omega = 0..2; the
channels of equal Omega couple through the variant's channel-pair j^2 term
(mod_Hphi_eCoriolis_01y2.f:901-911).  Bars as in the plain parity tests:
FP64 H psi <= 1e-12 relative, the norm trace, the recursion vectors and P(E)
<= 1e-10 after 150 iterations; the mixed path's H psi within 1e-6 of FP64.
"""
import ctypes as ct

import numpy as np
import pytest

from madwave3_gb300 import Propagator
from oracle.mw3ref import Oracle

pytestmark = pytest.mark.gpu
NIT = 150


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("ecor", [False, True])
def test_hphi_fp64(runs, ecor):
    """Lambda = 1 channels on the plain H, and the variant's coupling."""
    run = runs["tiny_ecor"]
    prop = Propagator(run, "fp64")
    prop.set_ecoriolis(ecor)
    ref = Oracle(run, ecoriolis=ecor)
    rng = np.random.default_rng(20261204)
    for _ in range(3):
        psi = rng.uniform(-1, 1, run.ntot)
        assert rel(prop.hphi(psi), ref.hphi(psi)) < 1e-12
    prop.close()


def test_coupling_is_exercised(runs):
    """The variant's H differs from the plain one by more than rounding."""
    run = runs["tiny_ecor"]
    psi = np.random.default_rng(5).uniform(-1, 1, run.ntot)
    a, b = Propagator(run, "fp64"), Propagator(run, "fp64")
    b.set_ecoriolis(True)
    ha, hb = a.hphi(psi), b.hphi(psi)
    assert np.abs(hb - ha).max() > 1e-3 * np.abs(ha).max()
    a.close()
    b.close()


def test_hphi_mixed(runs):
    run = runs["tiny_ecor"]
    p64, pmx = Propagator(run, "fp64"), Propagator(run, "mixed")
    p64.set_ecoriolis(True)
    pmx.set_ecoriolis(True)
    rng = np.random.default_rng(11)
    for _ in range(2):
        psi = rng.uniform(-1, 1, run.ntot)
        assert rel(pmx.hphi(psi), p64.hphi(psi)) < 1e-6
    p64.close()
    pmx.close()


def test_propagation_fp64(runs):
    run = runs["tiny_ecor"]
    prop = Propagator(run, "fp64")
    prop.set_ecoriolis(True)
    ref = Oracle(run, ecoriolis=True)
    prop.start()
    ref.start(run.psi0)
    prop.run(NIT)
    n_ref = ref.run_iters(NIT)
    assert rel(prop.norms()[1:], n_ref) < 1e-10
    km1, k, it = prop.state()
    rkm1, rk, rit = ref.state()
    assert it == rit == NIT + 1
    assert rel(k, rk) < 1e-10 and rel(km1, rkm1) < 1e-10
    p, pe = prop.totalflux()
    rp, rpe = ref.totalflux()
    assert rel(p, rp) < 1e-10 and rel(pe, rpe) < 1e-10
    prop.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_noalloc(runs, precision, tol):
    """mw3_hphi_noalloc applies the coupling as mw3_hphi does."""
    torch = pytest.importorskip("torch")
    run = runs["tiny_ecor"]
    prop = Propagator(run, precision)
    prop.set_ecoriolis(True)
    prop.L.mw3_hphi_noalloc.argtypes = [ct.c_void_p, ct.c_int32, ct.c_void_p, ct.c_void_p]
    prop.L.mw3_hphi_noalloc.restype = ct.c_int
    psi = np.random.default_rng(13).uniform(-1, 1, run.ntot)
    want = prop.hphi(psi)
    d_psi = torch.tensor(psi, dtype=torch.float64, device="cuda")
    d_out = torch.full_like(d_psi, float("nan"))
    torch.cuda.synchronize()
    rc = prop.L.mw3_hphi_noalloc(prop.h, 0, ct.c_void_p(d_psi.data_ptr()), ct.c_void_p(d_out.data_ptr()))
    assert rc == 0
    got = d_out.cpu().numpy()
    assert np.isfinite(got).all() and rel(got, want) <= tol
    prop.close()


def test_set_after_tables_exist_is_refused(runs):
    run = runs["tiny_ecor"]
    prop = Propagator(run, "fp64")
    prop.hphi(np.zeros(run.ntot))
    with pytest.raises(RuntimeError, match="mw3_set_ecoriolis"):
        prop.set_ecoriolis(True)
    prop.close()


def test_two_sources_per_target(runs):
    """tiny_ecor3 (Lambda = 0, 1, 0): every Lambda = 1 channel sums two sources
    in one CTA before its update of H."""
    run = runs["tiny_ecor3"]
    p64, pmx = Propagator(run, "fp64"), Propagator(run, "mixed")
    p64.set_ecoriolis(True)
    pmx.set_ecoriolis(True)
    ref = Oracle(run, ecoriolis=True)
    rng = np.random.default_rng(23)
    for _ in range(2):
        psi = rng.uniform(-1, 1, run.ntot)
        h = p64.hphi(psi)
        assert rel(h, ref.hphi(psi)) < 1e-12
        assert rel(pmx.hphi(psi), h) < 1e-6
    p64.close()
    pmx.close()
