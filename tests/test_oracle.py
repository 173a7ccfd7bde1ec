"""Known-answer and property tests of the CPU oracle (no GPU)."""
import numpy as np
import pytest
import scipy.fft
import scipy.special

from madwave3_gb300.host import constants as C
from oracle import mw3ref
from oracle.mw3ref import Oracle


@pytest.mark.parametrize("n", [1, 5, 24, 127, 128, 131, 256, 257, 384, 512])
def test_dst1_matches_definition_and_scipy(n):
    x = np.random.default_rng(n).standard_normal(n)
    ref = scipy.fft.dst(x, type=1)
    for mode in (0, 1):
        y = mw3ref.dst1(x, mode)
        assert np.abs(y - ref).max() <= 1e-13 * max(1.0, np.abs(ref).max())
    # RODFT00 applied twice is 2(n+1) times the identity
    yy = mw3ref.dst1(mw3ref.dst1(x, 0), 0)
    assert np.allclose(yy, 2 * (n + 1) * x, rtol=0, atol=1e-12 * n)


def test_noptfft_is_smallest_smooth():
    def smooth(v):
        for p in (2, 3, 5, 7, 11):
            while v % p == 0:
                v //= p
        return v == 1
    for ntot in (24, 128, 256):
        for nin in range(1, ntot + 1):
            n = mw3ref.noptfft(nin, ntot)
            assert n <= ntot
            cand = [m for m in range(nin, ntot + 1) if smooth(m)]
            assert n == (cand[0] if cand else ntot)


@pytest.mark.parametrize("l", [0, 1, 2, 5, 10, 25, 40])
def test_riccati_bessel(l):
    for x in (0.3, 1.0, 7.5, 25.0, 80.0, 250.0):
        f, g = mw3ref.riccati(l, x)
        fj = x * scipy.special.spherical_jn(l, x)
        gy = x * scipy.special.spherical_yn(l, x)
        assert f == pytest.approx(fj, rel=1e-10, abs=1e-300)
        if abs(gy) < 1e200:
            assert g == pytest.approx(gy, rel=1e-10)


@pytest.mark.parametrize("case", ["tiny_j0", "tiny_j3", "tiny_e2"])
def test_hamiltonian_symmetric(runs, case):
    run = runs[case]
    o = Oracle(run)
    rng = np.random.default_rng(7)
    a, b = rng.uniform(-1, 1, run.ntot), rng.uniform(-1, 1, run.ntot)
    ha, hb = o.hphi(a), o.hphi(b)
    assert abs(b @ ha - a @ hb) <= 1e-13 * abs(b @ ha)


@pytest.mark.parametrize("case", ["tiny_j3", "tiny_e2"])
def test_fft_and_direct_dst_agree_in_difs(runs, case):
    run = runs[case]
    psi = np.random.default_rng(3).uniform(-1, 1, run.ntot)
    h0 = Oracle(run, dst_mode=0).hphi(psi)
    h1 = Oracle(run, dst_mode=1).hphi(psi)
    assert np.abs(h0 - h1).max() <= 1e-13 * np.abs(h1).max()


def test_threaded_difs_matches_serial(runs):
    run = runs["tiny_j3"]
    psi = np.random.default_rng(5).uniform(-1, 1, run.ntot)
    h1 = Oracle(run, threads=1).hphi(psi)
    h4 = Oracle(run, threads=4).hphi(psi)
    assert np.abs(h1 - h4).max() <= 1e-13 * np.abs(h1).max()


def test_chebyshev_coefficients_closed_form(runs):
    run = runs["tiny_j0"]
    o = Oracle(run)
    et = o.flux_tables()["etot"]
    for k in (0, 1, 2, 17, 400):
        ck = o.coefecheby(k)
        es = (et - run.emindlt) / run.delta2
        d = 1.0 if k == 0 else 2.0
        ref = d * C.hbr / run.delta2 * np.exp(-1j * k * np.arccos(es)) / np.sqrt(1 - es * es)
        # the phase k*acos(Es) carries k ulps of argument rounding
        assert np.abs(ck - ref).max() <= 4e-16 * (k + 4) * np.abs(ref).max()


def test_propagation_deterministic_and_quirk_live(runs):
    run = runs["tiny_j0"]
    a, b = Oracle(run), Oracle(run)
    a.start(run.psi0)
    b.start(run.psi0)
    na, nb = a.run_iters(30), b.run_iters(30)
    assert np.array_equal(na, nb) and np.isfinite(na).all()
    # stored points beyond the r1 DST length exist in this grid: the quirk is exercised
    t = a.tables()
    beyond = sum(int((run.indr1[i, :run.npunreal[i]] > t["nopr1"][i]).sum()) for i in range(run.inp.nangu))
    assert beyond > 0


def test_quirk_points_keep_psi_as_kinetic_term(runs):
    """With V, the angular terms and the in-range kinetic term removed, H psi at a
    stored point beyond nopr1 is psi itself (mod_Hphi_01y2.f:818-831)."""
    run = runs["tiny_j0"]
    o = Oracle(run)
    t = o.tables()
    psi = np.zeros(run.ntot)
    # one quirk point, isolated
    for iang in range(1, run.inp.nangu + 1):
        n = run.npunreal[iang - 1]
        idx = np.nonzero(run.indr1[iang - 1, :n] > t["nopr1"][iang - 1])[0]
        if len(idx):
            ir = idx[0]
            break
    flat = run.offs[iang - 1, 0] + ir
    psi[flat] = 1.0
    h = o.hphi(psi)
    v = run.vvv[0, 0, iang - 1, ir]
    xj2 = o.xj2()[0, iang - 1, iang - 1, run.indr1[iang - 1, ir] - 1]
    xl2 = o.xl2p()[1, 0, iang - 1, iang - 1, run.indr2[iang - 1, ir] - 1]
    assert h[flat] == pytest.approx(1.0 + v + xj2 + xl2, rel=1e-14)


def test_norm_trace_of_the_damped_recursion(tmp_path, runs):
    """The check trace: without absorption psi_k = T_k(H_s) psi_0 with the scaled
    spectrum inside [-1, 1], so ||psi_k|| never exceeds ||psi_0||; with the
    absorbers the trace, oscillating from one iteration to the next as Chebyshev
    vectors do, decays once the packet reaches them."""
    import os
    from madwave3_gb300.host import generator, setup
    d = str(tmp_path / "undamped")
    generator.write_case(d, **dict(generator.CASES["tiny_j0"], absorb_strength=0.0))
    r0 = setup.load(os.path.join(d, "input.dat"))
    o = Oracle(r0)
    assert o.tables()["absfr1"].min() == 1.0 and o.tables()["absfr2"].min() == 1.0
    o.start(r0.psi0)
    n = o.run_iters(1500)
    assert n.max() <= float(np.sum(r0.psi0 ** 2)) * (1.0 + 1e-12)
    run = runs["tiny_j0"]
    o = Oracle(run, threads=4)
    o.start(run.psi0)
    n = o.run_iters(3000)
    assert n[-100:].mean() < 0.1 * n[:100].mean()
