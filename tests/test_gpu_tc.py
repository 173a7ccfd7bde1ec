"""tcgen05 tensor-core kernels of the mixed path: the 3xTF32 GEMM tile against
an FP64 product (through the library's self-test hook), and the factorised
angular contraction against the FP64 path and against separate runs."""
import ctypes as ct

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,N,K,bn", [(128, 128, 32, 128), (256, 256, 256, 256), (200, 256, 96, 256),
                                      (130, 100, 72, 128), (384, 512, 128, 256)])
def test_tc_gemm_tile(M, N, K, bn):
    torch = pytest.importorskip("torch")
    from madwave3_gb300 import load_library
    L = load_library()
    L.mw3_tc_gemm_selftest.argtypes = [ct.c_void_p] * 3 + [ct.c_int] * 4
    rng = np.random.default_rng(M * 7 + N + K)
    A = rng.standard_normal((M, K)).astype(np.float32)
    Bt = rng.standard_normal((N, K)).astype(np.float32)
    dA = torch.from_numpy(A).cuda()
    dB = torch.from_numpy(Bt).cuda()
    dC = torch.full((M, N), float("nan"), dtype=torch.float32, device="cuda")
    rc = L.mw3_tc_gemm_selftest(ct.c_void_p(dA.data_ptr()), ct.c_void_p(dB.data_ptr()), ct.c_void_p(dC.data_ptr()),
                                M, N, K, bn)
    assert rc == 0
    C = dC.cpu().numpy()
    ref = A.astype(np.float64) @ Bt.astype(np.float64).T
    err = np.abs(C - ref).max() / np.abs(ref).max()
    assert err < 5e-6, err          # FP32 accumulation over K <= 256


@pytest.mark.parametrize("case", ["tiny_j0", "tiny_j3", "tiny_e2"])
def test_fused_angular_runs_and_matches_fp64(runs, case):
    """The mixed path takes the tensor-core DSTs and the factorised tensor-core
    angular contraction, and its H psi agrees with FP64."""
    from madwave3_gb300 import Propagator

    run = runs[case]
    pmx = Propagator(run, "mixed")
    p64 = Propagator(run, "fp64")
    pmx.start()
    p64.start()
    pm, pf = pmx.path(), p64.path()
    assert pm["tc_dst"] and pm["tc_dst_fused"] and pm["tc_angular"], pm
    assert not any(pf.values()), pf
    rng = np.random.default_rng(7)
    psi = rng.uniform(-1.0, 1.0, run.ntot)
    a, b = pmx.hphi(psi), p64.hphi(psi)
    assert np.abs(a - b).max() / np.abs(b).max() < 1e-6
    pmx.close()
    p64.close()


def test_batched_waves_mixed(runs):
    """Waves with different block chains in one mixed context reproduce their
    separate mixed runs (every tile and chain is computed the same way)."""
    from madwave3_gb300 import Propagator

    r0, r3 = runs["tiny_j0"], runs["tiny_j3"]
    both = Propagator([r0, r3], "mixed")
    both.start()
    both.run(60)
    for w, r in enumerate((r0, r3)):
        one = Propagator(r, "mixed")
        one.start()
        one.run(60)
        x, y = both.state(w)[1], one.state()[1]
        assert np.abs(x - y).max() / np.abs(y).max() < 1e-12
        one.close()
    both.close()


@pytest.mark.parametrize("case", ["tiny_j0", "tiny_j3", "tiny_e2"])
def test_mixed_accumulators_track_fp64(runs, case):
    """After 150 iterations (four flushes of the FP32 rings and a partial one) the
    mixed path tracks the FP64 path: norms within 1e-5 and the flux and
    state-resolved accumulators (zCR, zCdR, zS2, Cvj) within 5e-4, relative to
    each quantity's largest magnitude, and P(E) within 1e-3 absolute (on these
    coarse grids, before the packet has passed the flux line, the mixed path's
    P(E) differs from FP64 by 2e-5 to 4e-4).  The case with two electronic
    states takes the update's several-source branch."""
    from madwave3_gb300 import Propagator

    run = runs[case]
    pmx = Propagator(run, "mixed")
    p64 = Propagator(run, "fp64")
    for p in (pmx, p64):
        p.start()
        p.run(150)
    rel = lambda a, b: np.abs(a - b).max() / max(np.abs(b).max(), 1e-300)
    assert rel(pmx.norms(), p64.norms()) < 1e-5
    assert np.abs(pmx.totalflux()[0] - p64.totalflux()[0]).max() < 1e-3
    am, a64 = pmx.accumulators(), p64.accumulators()
    for key in ("zcr", "zcdr", "zs2", "cvj"):
        assert np.abs(a64[key]).max() > 0, key
        assert rel(am[key], a64[key]) < 5e-4, key
    pmx.close()
    p64.close()


@pytest.mark.parametrize("case", ["tiny_j0", "tiny_e2"])
def test_regular_lines_match_general_tables(runs, case, monkeypatch):
    """When the flux lines' derivative terms are runs of consecutive points with
    consecutive r1, the mixed flux derivative reads the runs without per-term
    indices; MW3_GENERAL_TABLES=1 keeps the indexed form.  Both give the same bits."""
    from madwave3_gb300 import Propagator

    run = runs[case]
    out = []
    for general in ("0", "1"):
        monkeypatch.setenv("MW3_GENERAL_TABLES", general)
        p = Propagator(run, "mixed")
        p.start()
        p.run(40)
        out.append((p.state()[1], p.totalflux()[0], p.accumulators()["zcdr"]))
        p.close()
    for a, b in zip(out[0], out[1]):
        assert np.array_equal(a, b)


def test_state_all_round_trip(runs):
    """mw3_upload_state_all / mw3_download_state_all move every wave's state at
    once and agree with the per-wave calls."""
    from madwave3_gb300 import Propagator

    r0, r3 = runs["tiny_j0"], runs["tiny_j3"]
    p = Propagator([r0, r3], "mixed")
    p.start()
    p.run(5)
    km1, k, it = p.state_all()
    per = [p.state(w) for w in range(2)]
    assert np.array_equal(km1, np.concatenate([x[0] for x in per]))
    assert np.array_equal(k, np.concatenate([x[1] for x in per]))
    p.run(7)
    ref = p.state_all()[1]
    p.upload_state_all(km1, k, it)
    p.run(7)
    assert np.array_equal(p.state_all()[1], ref)
    p.close()


def test_transposed_rectangle_bit_identical(tmp_path, monkeypatch):
    """The FP32 rectangle stored [R][r1] (MW3_X_T=1: the update's stores coalesced
    along the stored points' r1 runs; the fused DST and the angular kernel read it
    that way) propagates bit for bit like the default [r1][R] layout: the same
    values reach the same operand positions."""
    import os
    from madwave3_gb300 import Propagator
    from madwave3_gb300.host import generator, setup

    d = str(tmp_path / "xt")
    generator.write_case(d, npun2=64, npun1=48, nangu=12, jmax=8, nvmax=2, netot=32, npun1min=8,
                         Jtot=2, iommax=2)
    run = setup.load(os.path.join(d, "input.dat"))
    out = {}
    for rect in ("0", "1"):
        monkeypatch.setenv("MW3_X_T", rect)
        p = Propagator(run, "mixed")
        p.start()
        path = p.path()
        assert path["tc_dst_fused"] and path["tc_angular"], path
        assert path["x_transposed"] == (rect == "1"), path
        p.run(40)
        out[rect] = (p.state()[1].copy(), p.norms().copy())
        psi = np.random.default_rng(48).uniform(-1.0, 1.0, run.ntot)
        out[rect + "h"] = p.hphi(psi)
        p.close()
    assert np.array_equal(out["0"][0], out["1"][0])
    assert np.array_equal(out["0"][1], out["1"][1])
    assert np.array_equal(out["0h"], out["1h"])
