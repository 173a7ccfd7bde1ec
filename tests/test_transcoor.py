"""ini_transcoor's set-up of the product projection (SRC/mod_coortrans01_02.f:
32-690) on the host: the reference's spline, the reactant -> product Jacobi
tables, and the whole set feeding the oracle's prodpaq / prodcvj."""
import math

import numpy as np

from madwave3_gb300.host import transcoor


def test_jordan_solves_the_spline_system():
    rng = np.random.default_rng(1)
    n = 9
    lam, mu, b = rng.uniform(0, 1, n), rng.uniform(0, 1, n), rng.standard_normal(n)
    A = np.diag(np.full(n, 2.0)) + np.diag(lam[1:], -1) + np.diag(mu[:-1], 1)
    assert np.allclose(transcoor.jordan(mu, lam, b), np.linalg.solve(A, b), atol=1e-13)


def test_spline_is_exact_for_cubics_and_accurate_for_smooth_functions():
    x = np.linspace(0.3, 4.0, 23)
    f = 0.5 - 1.5 * x + 0.7 * x ** 2 - 0.2 * x ** 3
    # four-point Lagrange derivative of a cubic is exact
    assert abs(transcoor.dlagra(x[:4], f[:4], 0) - (-1.5 + 1.4 * x[0] - 0.6 * x[0] ** 2)) < 1e-10
    d = transcoor.splset(f, x)
    for r in (0.31, 1.234, 2.5, 3.999):
        exact = 0.5 - 1.5 * r + 0.7 * r ** 2 - 0.2 * r ** 3
        assert abs(transcoor.splinqq(f, d, x, r) - exact) < 1e-11
    g = np.sin(x)
    dg = transcoor.splset(g, x)
    r = np.linspace(0.35, 3.95, 50)
    err = max(abs(transcoor.splinqq(g, dg, x, t) - math.sin(t)) for t in r)
    assert err < 2e-4


def test_dtrans(runs):
    """J = 0: all ones; Omega = Omega' = 0 at J = 3: d^3_00 = P_3 of the angle
    between the two R vectors."""
    r0 = runs["tiny_j0"]
    d0 = transcoor.dtrans(r0, 1.5, 3, 20, 2, 8, 0, 0)
    assert d0.shape == (r0.ncan, 1, 7, 18) and np.all(d0 == 1.0)
    r3 = runs["tiny_j3"]
    rb = 1.5
    d3 = transcoor.dtrans(r3, rb, 3, 20, 2, 8, 0, 2)
    inp = r3.inp
    a, bm = transcoor._ab(inp)
    b0 = [b for b in range(r3.ncan) if r3.iombas[b] == 0][0]
    checked = 0
    for ia, iang in enumerate(range(2, 9)):
        cg = r3.cgamma[iang - 1]
        for k, ir in enumerate(range(3, 21)):
            rga = inp.rmis2 + (ir - 1) * r3.ah2
            g = transcoor._geometry(inp, rga, cg, rb)
            if g is None:
                continue
            rpb = g[1]
            cb = (rb * rb + bm * bm * rpb * rpb - (rga * (inp.xm0 + inp.xm1) / inp.xm1) ** 2) * 0.5 / (bm * rpb * rb)
            if abs(cb) > 1:
                assert d3[b0, 0, ia, k] == 0
                continue
            ct = (bm * rpb * cb - rb) / math.sqrt((bm * rpb) ** 2 + rb * rb - 2 * bm * rpb * rb * cb)
            if abs(ct) > 1:
                continue
            p3 = 0.5 * (5 * ct ** 3 - 3 * ct)
            assert abs(d3[b0, 0, ia, k] - p3) < 1e-12
            checked += 1
    assert checked > 10


def test_trans_rg_jac(runs):
    run = runs["tiny_j3"]
    t = transcoor.trans_rg_jac(run, 1.5, 3, 7)
    blk, ang, r1, r2 = run.point_table()
    assert np.all(t[(ang < 3) | (ang > 7)] == 0)
    assert np.any(t != 0)
    # one point by the formula, written out
    inp = run.inp
    i = int(np.flatnonzero(t != 0)[len(np.flatnonzero(t != 0)) // 2])
    cg = run.cgamma[ang[i] - 1]
    rr2 = inp.rmis2 + (r2[i] - 1) * run.ah2
    rr1 = inp.rmis1 + (r1[i] - 1) * run.ah1
    a, _ = transcoor._ab(inp)
    c0 = (inp.xm0 + inp.xm2) * 1.5 / inp.xm2
    r1i = (rr2 * cg + math.sqrt(c0 * c0 + rr2 * rr2 * (cg * cg - 1))) / a
    n1 = inp.npun1
    s = sum(math.sin(math.pi * m / ((n1 + 1) * run.ah1) * rr1) * math.sin(math.pi * m / ((n1 + 1) * run.ah1) * r1i)
            for m in range(1, n1 + 1))
    jac = math.sqrt(1.5 * ((inp.xm0 + inp.xm2) / inp.xm2) ** 2 /
                    (a * math.sqrt(rr2 * rr2 * (cg * cg - 1) + (1.5 * (inp.xm0 + inp.xm2) / inp.xm2) ** 2)))
    assert abs(t[i] - s * 2 / (n1 + 1) * jac / math.sqrt(run.ah1)) < 1e-12 * max(1.0, abs(t[i]))


def _gauss_states(run, n2prod1, njp, nvp):
    """Normalised Gaussian radial functions standing in for the product diatom's."""
    x = run.inp.rmis2 + np.arange(n2prod1) * run.ah2
    out = np.zeros((njp, nvp, run.nelec, n2prod1))
    for jj in range(njp):
        for vv in range(nvp):
            g = np.exp(-((x - 1.2 - 0.1 * vv) / 0.25) ** 2) * (1 + 0.05 * jj)
            out[jj, vv, :, :] = g / math.sqrt(np.sum(g * g) * run.ah2)
    return out


def test_product_functions(runs):
    """prodwftrans is linear in the radial function (the spline is), and a
    product state with j' below |Omega'| has no Wigner component."""
    run = runs["tiny_j3"]
    st = _gauss_states(run, 30, 2, 1)
    f1, f2 = st[0, 0], st[1, 0] * 0.3 + 0.01 * np.arange(30)[None, :]
    pa = transcoor.prod_functions(run, 1.5, f1, 3, 30, 2, 8, 1, 2, 0)
    pb = transcoor.prod_functions(run, 1.5, f2, 3, 30, 2, 8, 1, 2, 0)
    pab = transcoor.prod_functions(run, 1.5, 2.0 * f1 - f2, 3, 30, 2, 8, 1, 2, 0)
    assert np.any(pa != 0) and np.all(np.isfinite(pa))
    assert np.allclose(pab, 2.0 * pa - pb, rtol=0, atol=1e-12 * np.abs(pa).max())
    assert np.all(transcoor.prod_functions(run, 1.5, f1, 3, 30, 2, 8, 2, 1, 0) == 0)


def test_vectorised_product_functions_match_the_pointwise_ones(runs):
    """ini_transcoor's prodwftrans over all (angle, R) points at once gives the
    point-by-point restatement's numbers for every state of an Omega."""
    run = runs["tiny_j3"]
    jp0, jp1, vp0, vp1 = 0, 3, 0, 1
    nob = np.array([1, 1, 0, 1], np.int32)
    fd = _gauss_states(run, 30, jp1 - jp0 + 1, vp1 - vp0 + 1)
    for iom in (0, 1, 2):
        allv = transcoor.prod_functions_omega(run, 1.5, fd, nob, jp0, jp1, vp0, 3, 30, 2, 8, iom)
        for j in range(jp0, jp1 + 1):
            for iv in range(vp0, int(nob[j - jp0]) + 1):
                one = transcoor.prod_functions(run, 1.5, fd[j - jp0][iv - vp0], 3, 30, 2, 8, iom, j, iv)
                got = allv[j - jp0, iv - vp0]
                assert np.allclose(got, one, rtol=0, atol=1e-14 * max(np.abs(one).max(), 1e-300)), (iom, j, iv)


def test_ini_transcoor_feeds_the_oracle_projection(runs):
    from oracle.mw3ref import Oracle

    run = runs["tiny_j3"]
    jp0, jp1, vp0, vp1 = 0, 3, 0, 1
    nob = np.array([1, 1, 0, 1], np.int32)
    fd = _gauss_states(run, 30, jp1 - jp0 + 1, vp1 - vp0 + 1)
    pp = transcoor.ini_transcoor(run, 1.5, 3, 30, 2, 8, 0, 2, jp0, jp1, vp0, vp1, nob, fd)
    assert pp.prodwf.shape == (3, 4, 2, run.nelec, 7, 28)
    assert np.all(pp.prodwf[1, 0] == 0) and np.all(pp.prodwf[2, :2] == 0)     # j < Omega
    o = Oracle(run)
    o.set_product(pp)
    o.start(run.psi0)
    o.run_iters(20)
    z, c = o.product()
    assert np.all(np.isfinite(z)) and np.any(z != 0)
    fac = transcoor.s2prodfac(run, o.flux_tables()["etot"], o.flux_tables()["apaqini"],
                              np.full((4, 2), -0.1), nob, vp0, vp1)
    assert fac.shape == (4, 2, run.inp.netot) and np.all(fac >= 0) and np.any(fac > 0)
    assert np.all(fac[2, 1] == 0)                                                # v > noBCprod(j)


def test_product_chain_from_the_generator_to_the_probability_file(runs, tmp_path):
    """Synthetic product states (the 02 diatom of the LEPS surface) -> the
    ini_transcoor tables -> the oracle's prodpaq / prodcvj -> printprob's
    iprod = 2 S2prod with S2prodfac from the states' energies."""
    from madwave3_gb300 import printprob
    from madwave3_gb300.host import generator
    from oracle.mw3ref import Oracle

    run = runs["tiny_j3"]
    over = generator.CASES["tiny_j3"]
    fd, ed, nob = generator.product_states(run, 30, 0, 4, 0, 2, **over)
    assert fd.shape == (5, 3, run.nelec, 30) and np.all(nob >= 0)
    # lowest state: discrete-normalised over the whole grid, so at most 1 on 30 points
    assert 0.5 < np.sum(fd[0, 0] ** 2) <= 1.0 + 1e-12
    assert np.all(np.diff(ed[0]) > 0) and np.all(ed[1:, 0] > ed[:-1, 0])        # v and j ladders
    pp = transcoor.ini_transcoor(run, 1.8, 3, 30, 1, run.inp.nangu, 0, 2, 0, 4, 0, 2, nob, fd)
    o = Oracle(run)
    o.set_product(pp)
    o.start(run.psi0)
    o.run_iters(30)
    z, _ = o.product()
    ft = o.flux_tables()
    fac = transcoor.s2prodfac(run, ft["etot"], ft["apaqini"], ed, nob, 0, 2)
    zs2, _ = o.s2()
    path = printprob.write_s2prod(str(tmp_path), run, 1, *o.totalflux(), zs2, ft["etot"], ft["reacfct"],
                                  o.s2factor(), iprod=2, product=(z, fac, pp))
    a = printprob.read_s2prod(path)
    assert a.shape == (run.inp.netot, 4 + 3)
    assert np.all(np.isfinite(a)) and np.all(a[:, 3:] >= 0) and np.any(a[:, 3] > 0)
