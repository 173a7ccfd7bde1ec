"""mw3_hphi_noalloc: H psi with no allocation, through the C-ABI.

The entry point serves callers that may allocate GPU memory only at start-up
(a host whose device memory belongs to another allocator, or a time loop that
must not pay cudaMalloc's implicit synchronisation).  Its scratch is one
static device array shared by every call, so two calls in a row must both
agree with mw3_hphi: the second call proves the array's leftover contents
from the first call do not leak into the result.  This file is named to be
collected last.
"""
import ctypes as ct
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MW3_ERR_ARG, MW3_ERR_UNSUPPORTED, MW3_ERR_STATE = 1, 3, 4


def _rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def _bind(lib):
    lib.mw3_hphi_noalloc.argtypes = [ct.c_void_p, ct.c_int32, ct.c_void_p, ct.c_void_p]
    lib.mw3_hphi_noalloc.restype = ct.c_int


def _noalloc(torch, prop, wave, psi):
    d_psi = torch.tensor(psi, dtype=torch.float64, device="cuda")
    d_out = torch.full_like(d_psi, float("nan"))
    torch.cuda.synchronize()
    rc = prop.L.mw3_hphi_noalloc(prop.h, wave, ct.c_void_p(d_psi.data_ptr()), ct.c_void_p(d_out.data_ptr()))
    assert rc == 0, prop.L.mw3_last_error(prop.h)
    return d_out.cpu().numpy()


# tolerances as in the parity tests: FP64 1e-12; mixed 1e-6 (FP32 transforms, and
# mw3_hphi takes its radial DSTs on the tensor cores where this entry point does not)
@pytest.mark.parametrize("case,precision,tol", [("tiny_j3", "fp64", 1e-12), ("tiny_e2", "mixed", 1e-6)])
def test_hphi_noalloc_matches_hphi(runs, case, precision, tol):
    torch = pytest.importorskip("torch")
    from madwave3_gb300 import Propagator

    run = runs[case]
    prop = Propagator(run, precision)
    _bind(prop.L)
    rng = np.random.default_rng(20261203)
    psis = [rng.uniform(-1.0, 1.0, run.ntot), rng.uniform(-1.0, 1.0, run.ntot)]
    for psi in psis:                       # two calls in a row, different inputs
        expected = prop.hphi(psi)          # the existing entry point (host arrays)
        got = _noalloc(torch, prop, 0, psi)
        assert np.isfinite(got).all()
        assert _rel(got, expected) <= tol
    prop.close()


@pytest.mark.parametrize("precision,tol", [("fp64", 1e-12), ("mixed", 1e-6)])
def test_hphi_noalloc_second_wave(case_dirs, precision, tol):
    """A later wave of a batch: its blocks and flat offsets start after the
    first wave's, so the entry point's shifted bases are exercised."""
    torch = pytest.importorskip("torch")
    from madwave3_gb300 import Propagator
    from madwave3_gb300.host import generator, setup

    waves = setup.load_sweep(os.path.join(case_dirs["tiny_j0"], "input.dat"), [1, 2], generator.jsweep_inputs)
    prop = Propagator(waves, precision)
    _bind(prop.L)
    rng = np.random.default_rng(7)
    for _ in range(2):
        psi = rng.uniform(-1.0, 1.0, waves[1].ntot)
        expected = prop.hphi(psi, wave=1)
        got = _noalloc(torch, prop, 1, psi)
        assert _rel(got, expected) <= tol
    prop.close()


def test_hphi_noalloc_rejections(runs, tmp_path):
    """Before the device tables exist: MW3_ERR_STATE; overlapping psi/hpsi:
    MW3_ERR_ARG; a wave whose scratch exceeds the static array: MW3_ERR_UNSUPPORTED.
    Each is refused before anything is launched."""
    torch = pytest.importorskip("torch")
    from madwave3_gb300 import Propagator
    from madwave3_gb300.host import generator, setup

    run = runs["tiny_j0"]
    prop = Propagator(run, "fp64")
    _bind(prop.L)
    d = torch.zeros(2 * run.ntot, dtype=torch.float64, device="cuda")
    p0 = d.data_ptr()
    assert prop.L.mw3_hphi_noalloc(prop.h, 0, ct.c_void_p(p0), ct.c_void_p(p0 + 8 * run.ntot)) == MW3_ERR_STATE
    prop.hphi(np.zeros(run.ntot))                          # builds the device tables
    assert prop.L.mw3_hphi_noalloc(prop.h, 0, ct.c_void_p(p0), ct.c_void_p(p0 + 8)) == MW3_ERR_ARG
    assert prop.L.mw3_hphi_noalloc(prop.h, 0, ct.c_void_p(p0), ct.c_void_p(p0)) == MW3_ERR_ARG
    assert prop.L.mw3_hphi_noalloc(prop.h, 5, ct.c_void_p(p0), ct.c_void_p(p0 + 8 * run.ntot)) == MW3_ERR_ARG
    prop.close()
    # 256 x 256 x 72 rectangle of FP64: 36 MiB per scratch rectangle, two needed
    big = str(tmp_path / "big")
    generator.write_case(big, npun2=256, npun1=256, nangu=72, jmax=10, nvmax=1, netot=8, npun1min=32)
    brun = setup.load(os.path.join(big, "input.dat"))
    bprop = Propagator(brun, "fp64")
    _bind(bprop.L)
    bprop.hphi(np.zeros(brun.ntot))
    dd = torch.zeros(2 * brun.ntot, dtype=torch.float64, device="cuda")
    rc = bprop.L.mw3_hphi_noalloc(bprop.h, 0, ct.c_void_p(dd.data_ptr()),
                                  ct.c_void_p(dd.data_ptr() + 8 * brun.ntot))
    assert rc == MW3_ERR_UNSUPPORTED
    assert b"scratch" in bprop.L.mw3_last_error(bprop.h)
    bprop.close()
