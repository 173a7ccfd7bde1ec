"""Product diatom states of uncoupled electronic states (the diabatic_prod_pot
= 0 branch of product_radialf_write, bndbc1ele) on Morse potentials, whose
levels are known in closed form, and the func/prodwf file they are written to."""
import math
import os
from types import SimpleNamespace

import numpy as np

from madwave3_gb300.host import constants as C
from madwave3_gb300.host import potini, setup

A, RE = 1.03, 1.4                           # bohr^-1, bohr
MORSE = [(0.17, 0.0), (0.12, 0.02)]         # (De, asymptote) of each state, hartree
MU = 918.6                                  # a.u.


def potelebond(r1, r2, ctet):
    v = np.zeros((len(MORSE), len(MORSE), len(r2)))
    for k, (de, top) in enumerate(MORSE):
        v[k, k] = de * (1.0 - np.exp(-A * (r2 - RE))) ** 2 - de + top
    return v


def morse_level(k, v):
    de, top = MORSE[k]
    w = A * math.sqrt(2.0 * de / MU)
    return top - de + w * (v + 0.5) - w * w / (4.0 * de) * (v + 0.5) ** 2


def grid(n2prod1=600):
    rmis2, rfin2 = 0.1 * C.convl, 15.0 * C.convl            # angstrom
    g = SimpleNamespace(inp=SimpleNamespace(rmis2=rmis2, rfin2=rfin2, npun2=1024), xm1prod=MU / C.convm)
    g.ah2 = (rfin2 - rmis2) / 1023.0
    return g, n2prod1


def test_levels_order_and_normalisation():
    g, n2p = grid()
    fd, e, nob, elec, vib = potini.product_radialf_write_adiabatic(
        g, potelebond, 0, 7, 0, 0, n2p, nelec=2, max_viblevels=[5, 3])
    # state 1's five levels, then state 2's three, in that order (not sorted by energy)
    assert nob[0] == 7
    assert list(elec[0]) == [1] * 5 + [2] * 3 and list(vib[0]) == [0, 1, 2, 3, 4, 0, 1, 2]
    want = [morse_level(0, v) for v in range(5)] + [morse_level(1, v) for v in range(3)]
    got = e[0] / C.conve1 * C.conve                         # zot -> hartree
    assert np.allclose(got, want, rtol=1e-6, atol=0)
    # each function lives in its own state and is discrete-normalised
    for k in range(8):
        own = elec[0, k] - 1
        assert abs(np.sum(fd[0, k, own] ** 2) - 1.0) < 1e-10
        assert not fd[0, k, 1 - own].any()


def test_rotation_raises_the_levels_and_nvini_numbers():
    g, n2p = grid()
    _, e0, _, _, _ = potini.product_radialf_write_adiabatic(g, potelebond, 0, 3, 0, 4, n2p)
    assert np.all(np.diff(e0[:, 0]) > 0)                   # v = 0 rises with j
    _, e1, nob1, _, vib1 = potini.product_radialf_write_adiabatic(g, potelebond, 1, 3, 0, 0, n2p,
                                                                  max_viblevels=[4])
    # the count starts at nvini - 1, so nvini numbers the state's v = 0 (nothing is
    # skipped); of its four levels the fourth, numbered 4 > nvmaxprod, is dropped
    assert list(vib1[0]) == [0, 1, 2] and np.allclose(e1[0], e0[0, :3], rtol=1e-12) and nob1[0] == 3


def test_prodwf_file_round_trip(tmp_path):
    g, n2p = grid(200)
    fd, e, nob, elec, vib = potini.product_radialf_write_adiabatic(
        g, potelebond, 0, 5, 0, 1, n2p, nelec=2, max_viblevels=[4, 2])
    potini.write_prodwf(str(tmp_path), 0, 0, fd, e, nob, elec, vib)
    f2, e2, n2, el2, vb2 = setup.product_radialf_read(os.path.join(str(tmp_path), "func", "prodwf"), 0, 1, 0, 5, n2p,
                                                      eref=0.25)
    assert np.array_equal(n2, nob) and np.array_equal(el2, elec) and np.array_equal(vb2, vib)
    assert np.array_equal(f2, fd) and np.allclose(e2, e - 0.25, rtol=0, atol=1e-15)


# ---- several coupled electronic states: pot1 and the product box DVR ----

def two_state_surface(x1, x2, calpha):
    """A two-state diabatic surface in hartree, smooth in the bond coordinates."""
    x1, x2, calpha = np.asarray(x1), np.asarray(x2), np.asarray(calpha)
    v1 = 0.17 * (1.0 - np.exp(-A * (x1 - RE))) ** 2 - 0.17 + 0.05 * np.exp(-0.5 * (x2 - 2.0) ** 2)
    v2 = v1 + 0.03 + 0.01 * calpha
    c = 0.004 * np.exp(-0.3 * (x2 - 2.5) ** 2)
    return np.array([[v1, c], [c, v2]])


def small_grid(n1=12, n2=16, na=4):
    from madwave3_gb300.host import generator
    groups, _ = generator.make_inputs(npun1=n1, npun2=n2, nangu=na, nelecmax=2, jmax=3, nvmax=1, npun1min=4)
    inp, _ = potini._inputs(groups)
    return potini._grid(inp)


def test_pot1_coupled_states(tmp_path):
    g = small_grid()
    i = g.inp
    vref = -0.05
    npunreal, vmin, vmaxtot = potini.pot1(g, two_state_surface, vref, str(tmp_path), nelec=2,
                                          states=[(0, 0, 1.0, 1.0), (1, 0, 1.0, 1.0)])
    lines = open(os.path.join(str(tmp_path), "pot", "cont.pot")).read().splitlines()
    assert lines[0].split() == ["2"] and lines[2].split()[:2] == ["1", "0"]
    gam = i.xm1 / (i.xm0 + i.xm1)
    seen_min = 1e10
    for a in range(i.nangu):
        rows = np.loadtxt(os.path.join(str(tmp_path), "pot", "pot.%03d.dat" % (a + 1)), ndmin=2)
        assert len(rows) == npunreal[a]
        stored = {(int(r[0]), int(r[1])): r[2:] for r in rows}
        for ir2 in range(1, i.npun2 + 1):
            for ir1 in range(1, i.npun1 + 1):
                rp = (i.rmis1 + (ir1 - 1) * g.ah1) / C.convl
                rg = (i.rmis2 + (ir2 - 1) * g.ah2) / C.convl
                ct = float(g.cgamma[a])
                x2 = math.sqrt(rg * rg + gam * gam * rp * rp + 2.0 * gam * rg * rp * ct)
                ca = max(-1.0, min(1.0, (rg * ct + gam * rp) / x2))
                m = two_state_surface(rp, x2, ca) / C.conve * C.conve1
                m[0, 0] -= vref
                m[1, 1] -= vref
                for e in range(2):
                    if m[e, e] > g.vcutmax:
                        m[e, :] = 0.0
                        m[:, e] = 0.0
                        m[e, e] = g.vcutmax
                w = np.linalg.eigvalsh(m)
                seen_min = min(seen_min, w.min())
                if (w < g.vcutmax).any():
                    # the matrix column by column (V11 V21 V12 V22)
                    assert np.allclose(stored[(ir1, ir2)], m.T.ravel(), rtol=1e-12, atol=1e-15)
                else:
                    assert (ir1, ir2) not in stored
    assert abs(vmin - seen_min) <= 1e-12 * abs(seen_min) and vmaxtot >= g.vcutmax


def test_coupled_product_levels():
    g, _ = grid()
    n = g.inp.npun2

    def uncoupled(r1, r2, ctet):
        v = potelebond(r1, r2, ctet)
        return v                                          # no off-diagonal terms

    fd, e, nob, = potini.product_radialf_write(g, uncoupled, 0, 5, 0, 0, n, nelec=2)
    singles = []
    for k in range(2):
        one = lambda r1, r2, ct, k=k: potelebond(r1, r2, ct)[k:k + 1, k:k + 1]
        singles.extend(potini.product_radialf_write(g, one, 0, 5, 0, 0, n)[1][0])
    assert np.allclose(e[0], np.sort(singles)[:6], rtol=1e-10)
    elec, vib = potini.product_labels(fd, 0)
    assert list(vib[0]) == list(range(6)) and set(elec[0]) <= {1, 2}

    def coupled(r1, r2, ctet):
        v = potelebond(r1, r2, ctet)
        v[0, 1] = v[1, 0] = 0.003 * np.exp(-(r2 - RE) ** 2)
        return v

    fd, e, nob = potini.product_radialf_write(g, coupled, 0, 5, 0, 0, n, nelec=2)
    assert np.all(np.diff(e[0]) > 0) and list(nob) == [5]
    # n2prod1 = npun2: each level is normalised over both states
    assert np.allclose(np.sum(fd[0] ** 2, axis=(1, 2)), 1.0, rtol=1e-10)


def test_two_state_case_through_the_readers(tmp_path):
    """pot.out for a two-state surface with adiabatic products (the current
    source's default form): the main program's readers load the case and the
    oracle applies H to it."""
    from madwave3_gb300.host import generator, namelist
    from oracle.mw3ref import Oracle
    groups, _ = generator.make_inputs(npun1=16, npun2=24, nangu=6, nelecmax=2, jmax=3, nvmax=1, npun1min=4,
                                      netot=16, Jtot=0, alpha0_bohr=1.2)
    groups["inputprod"] = dict(iprod=2, nviniprod=0, nvmaxprod=2, jiniprod=0, jmaxprod=2, iomminprod=0,
                               iommaxprod=0, rbalinprod=3.0, n2prod0=2, n2prod1=20, nangproj0=1, nangproj1=6)
    d = str(tmp_path / "case")
    out = potini.write_case(d, None, two_state_surface, input_text=namelist.dumps(groups), product_form="namelist",
                            states=[(0, 0, 1.0, 1.0), (0, 0, 1.0, 1.0)])
    assert out["npunreal"].sum() > 0 and out["nobc"].shape[0] == 2
    run = setup.load(os.path.join(d, "input.dat"))
    assert run.nelec == 2 and run.ntot > 0
    psi = np.random.default_rng(2).uniform(-1, 1, run.ntot)
    assert np.all(np.isfinite(Oracle(run).hphi(psi)))
    fdp, edp, nobp = out["product"]
    f2, e2, n2, el2, vb2 = setup.product_radialf_read(os.path.join(d, "func", "prodwf"), 0, 2, 0, 2, 20)
    assert np.array_equal(n2, nobp) and np.allclose(e2, edp, rtol=1e-15, atol=0)
    assert set(np.unique(el2[el2 > 0])) <= {1, 2}
