"""CRP-fast (SRC/AUXILIARy-CODES/CRP-fast.f) restated: J-shifted cumulative
reaction probabilities from distriS2prod tables, checked where the answer is
known in closed form, and the program end to end on the files distri writes."""
import os

import numpy as np
import pytest

from madwave3_gb300 import crp, distri
from madwave3_gb300.host import namelist

E_TAB = np.linspace(0.1, 1.5, 60)          # eV: the tables' energies


def flat_tables(jcalc, jref, nv, nj, f):
    """Every calculated J (J >= |Omega|) holds S2 = f(E, v, j)."""
    out = {}
    for om in range(-jref, jref + 1):
        for J in jcalc:
            if J < abs(om):
                continue
            for iv in range(nv):
                s2 = np.stack([f(E_TAB, iv, j) for j in range(nj)], axis=1)
                out[(om, J, iv, 1)] = (E_TAB, s2)
    return out


def weight(J, om, jc):
    """The share of the common table a J takes without shifts: 1 at and above
    the last calculated J, else the linear interpolation between the calculated
    J around it, a calculated J below |Omega| counting as zeros (it has no table)."""
    if J >= jc[-1]:
        return 1.0
    j1 = max(x for x in jc if x <= J)
    j2 = jc[jc.index(j1) + 1]
    w1, w2 = float(j1 >= abs(om)), float(j2 >= abs(om))
    return w1 if J == j1 else ((j2 - J) * w1 + (J - j1) * w2) / (j2 - j1)


def test_unshifted_sum_is_closed_form():
    """B_J = 0 and the same table for every calculated J: CRP = sum_J (2J+1) w_J S2."""
    jc, jtotmax, jref = [0, 3, 7], 10, 1
    f = lambda e, v, j: 0.2 + 0.1 * v + 0.05 * j + 0.3 * e ** 2
    tabs = flat_tables(jc, jref, 2, 3, f)
    eg = np.linspace(0.2, 1.4, 25)
    out, pj = crp.crp(tabs, jc, {J: 0.0 for J in jc}, jtotmax, jref, eg, 0, 1, 1, 3)
    for om in range(-jref, jref + 1):
        w = sum((2 * J + 1) * weight(J, om, jc) for J in range(abs(om), jtotmax + 1))
        for iv in range(2):
            for j in range(3):
                assert np.allclose(out[:, j, iv, 0, om + jref], w * f(eg, iv, j), rtol=1e-12)
    # P_J sums every state and every Omega that reaches J
    want = sum(f(eg, v, j) for v in range(2) for j in range(3))
    for J in range(jtotmax + 1):
        share = sum(weight(J, om, jc) for om in range(-jref, jref + 1) if abs(om) <= J)
        assert np.allclose(pj[:, J], share * want, rtol=1e-12)


def test_j_shifting_of_linear_tables():
    """A linear S2 is reproduced by the spline, so J shifting is the closed form
    [(J2 - J) S(E - B1 (J(J+1) - J1(J1+1))) + (J - J1) S(E + B2 (J2(J2+1) - J(J+1)))] / (J2 - J1),
    0 below the table's grid and its last value above."""
    jc, jtotmax = [0, 4, 8], 12
    be = {0: 0.002, 4: 0.0015, 8: 0.001}
    f = lambda e, v, j: 0.1 + 0.4 * e
    tabs = flat_tables(jc, 0, 1, 1, f)
    eg = np.linspace(0.3, 1.3, 21)

    def lin(e):
        return np.where(e < E_TAB[0], 0.0, np.where(e > E_TAB[-1], f(E_TAB[-1], 0, 0), f(e, 0, 0)))

    out, _ = crp.crp(tabs, jc, be, jtotmax, 0, eg, 0, 0, 1, 1)
    want = np.zeros(len(eg))
    for J in range(jtotmax + 1):
        if J >= jc[-1]:
            s = lin(eg - be[8] * (J * (J + 1) - 72))
        else:
            j1 = max(x for x in jc if x <= J)
            j2 = jc[jc.index(j1) + 1]
            s1 = lin(eg - be[j1] * (J * (J + 1) - j1 * (j1 + 1)))
            s2 = lin(eg + be[j2] * (j2 * (j2 + 1) - J * (J + 1)))
            s = s1 if J == j1 else ((j2 - J) * s1 + (J - j1) * s2) / (j2 - j1)
        want += (2 * J + 1) * s
    assert np.allclose(out[:, 0, 0, 0, 0], want, rtol=1e-12)


def test_below_the_first_calculated_j_is_refused():
    tabs = flat_tables([2, 5], 0, 1, 1, lambda e, v, j: e)
    with pytest.raises(ValueError, match="below the first calculated J"):
        crp.crp(tabs, [2, 5], {2: 0.0, 5: 0.0}, 6, 0, np.array([0.5]), 0, 0, 1, 1)


def test_table_directories():
    assert crp.table_dir("b", 0, 7) == os.path.join("b", "Omg0", "J007")
    assert crp.table_dir("b", 1, 4) == os.path.join("b", "Omg1", "p", "J004")
    assert crp.table_dir("b", 1, 5) == os.path.join("b", "Omg1", "m", "J005")
    assert crp.table_dir("b", -1, 4) == os.path.join("b", "Omg1", "m", "J004")
    assert crp.table_dir("b", -1, 5) == os.path.join("b", "Omg1", "p", "J005")


def test_program_on_distri_files(tmp_path):
    """distriS2prod files as distri writes them for J = 0, 2, 5 (jref = 0), read by
    the program: with B_J = 0 its CRPtot is the closed-form sum."""
    nv, nj, netot = 2, 3, 40
    e_zot = distri.energy_grid(0.1, 1.5, netot)
    e_ev = e_zot / (distri.CONVE1 * distri.EV2CM)
    jc = [0, 2, 5]
    for J in jc:
        d = tmp_path / "Omg0" / ("J%03d" % J)
        d.mkdir(parents=True)
        vibrot = np.stack([np.stack([(0.1 + 0.05 * v + 0.02 * j) * (1 + e_ev) for j in range(nj)], axis=1)
                           for v in range(nv)])
        distri.write_files(str(d), e_zot, vibrot, vibrot.sum(axis=2), vibrot.sum(axis=(0, 2)), 0)
    work = tmp_path / "sigma"
    work.mkdir()
    (work / "CalculatedJ.dat").write_text("".join("%d 0.0\n" % J for J in jc))
    groups = {
        "inputgridbase": dict(jref=0, jini=0, jmax=3, nvini=0, nvmax=1, nelecmax=1),
        "inputprod": dict(iprod=2, nviniprod=0, nvmaxprod=nv - 1, jiniprod=0, jmaxprod=nj - 1),
        "inputpotmass": dict(xm0=2.014, xm1=1.008, xm2=1.008),
        "inputflux": dict(netot=netot),
        "sigmas2prod": dict(jtotmax=7, ncalc=len(jc), nesigma=15, eminsigma_ev=0.3, emaxsigma_ev=1.2),
    }
    (work / "input.dat").write_text(namelist.dumps(groups))
    eg, out, pj = crp.run_program(str(work))
    tot = np.loadtxt(str(work / "CRPtot.res"), comments="#")
    assert tot.shape == (15, 3)
    w = sum(2 * J + 1 for J in range(8))
    want = w * sum((0.1 + 0.05 * v + 0.02 * j) * (1 + eg) for v in range(nv) for j in range(nj))
    # the distri files carry 8 significant digits (e15.7)
    assert np.allclose(tot[:, 2], want, rtol=1e-6)
    assert np.allclose(tot[:, 1], crp.k2(eg, 1.008 * 3.022 / 4.03), rtol=1e-6)
    vib = np.loadtxt(str(work / "CRPvib.res"))
    assert vib.shape == (15, 2 + nv) and np.allclose(vib[:, 2:].sum(axis=1), tot[:, 2], rtol=1e-6)
    assert os.path.exists(str(work / "CRP.vf01.ef1")) and np.loadtxt(str(work / "PJ.res")).shape == (15, 9)
