"""Cumulative reaction probabilities from the state-resolved product
distributions, as the post-processing program CRP-fast does
(SRC/AUXILIARy-CODES/CRP-fast.f).

Input: for each reactant Omega (iomref0 = -jref..jref), product vibrational
level v and electronic state, the files distriS2prod.vVV.eE (E in eV, then
S2 for each product j; madwave3_gb300.distri) of the calculated total J,
found as ../OmgN/JXXX (Omega = 0) or ../OmgN/{p,m}/JXXX (the parity subfolder
p for Omega > 0 and even J or Omega < 0 and odd J, else m), the list of
calculated J with their J-shifting rotational constants B_J (eV) in
CalculatedJ.dat, and the namelists of input.dat (the &sigmaS2prod group:
Jtotmax, nCalc, nESigma, EminSigma_eV, EmaxSigma_eV).

For every J from |Omega| to Jtotmax, each product (v, j) column is brought to
the output grid E_i = Emin + (i - 1) (Emax - Emin) / (nESigma - 1) by J
shifting (:241-380): between calculated J1 < J < J2,
    S2_J(E) = [(J2 - J) S2_J1(E - B_J1 (J(J+1) - J1(J1+1))) + (J - J1) S2_J2(E + B_J2 (J2(J2+1) - J(J+1)))] / (J2 - J1),
at a calculated J its own values, above the last one that one shifted; each
S2 is the reference's spline of a calculation's column, 0 below its energy
grid and its last value above it, and negative results are set to 0.  Then
    CRP(E; j, v, e, Omega) = sum_J (2J + 1) S2_J(E),   P_J(E) = sum S2_J(E)
over every state, and the files CRPtot.res, CRPvib.res, CRPomg.res, PJ.res
and CRP.vfVV.efE with k^2 = 2 mu E / hbar^2 (E in zot, mu the reactant
arrangement's for iprod = 2) beside each energy (:400-480).
"""
import os

import numpy as np

from .sigma import _shifted

# CRP-fast.f:50-58
CONVE1 = 1.197e-4
HBR = 0.063533625
CEVCM = 1.23984245e-4


def table_dir(base, iomref0, Jtot):
    """The directory of one calculated J for one reactant Omega (:190-235)."""
    a = abs(iomref0)
    if iomref0 == 0:
        return os.path.join(base, "Omg%d" % a, "J%03d" % Jtot)
    parity = "p" if (iomref0 > 0) == (Jtot % 2 == 0) else "m"
    return os.path.join(base, "Omg%d" % a, parity, "J%03d" % Jtot)


def read_calculated_j(path, ncalc):
    """(Jcalc, {J: B_J in eV}) from CalculatedJ.dat (:157-170)."""
    jc, be = [], {}
    with open(path) as f:
        for _ in range(ncalc):
            t = f.readline().split()
            jc.append(int(t[0]))
            be[int(t[0])] = float(t[1].replace("D", "E"))
    return jc, be


def read_tables(base, jcalc, jref, nv0, nv1, nel, nener):
    """{(Omega, J, v, e): (E[nener] eV, S2[nener][nj])} of the calculated J with
    J >= |Omega| (:186-239)."""
    out = {}
    for om in range(-jref, jref + 1):
        for J in jcalc:
            if J < abs(om):
                continue
            for iv in range(nv0, nv1 + 1):
                for ie in range(1, nel + 1):
                    a = np.loadtxt(os.path.join(table_dir(base, om, J), "distriS2prod.v%02d.e%d" % (iv, ie)),
                                   ndmin=2)[:nener]
                    out[(om, J, iv, ie)] = (a[:, 0], a[:, 1:])
    return out


def _column(tab, key, j, egrid, shift):
    if key not in tab:
        return np.zeros(len(egrid))
    e, s2 = tab[key]
    return _shifted(e, s2[:, j], egrid, shift)


def crp(tables, jcalc, be, jtotmax, jref, egrid, nv0, nv1, nel, nj):
    """CRP[nE][nj][nv][nel][2 jref + 1] and PJ[nE][Jtotmax + 1] (:171-384)."""
    jc = sorted(jcalc)
    ne = len(egrid)
    out = np.zeros((ne, nj, nv1 - nv0 + 1, nel, 2 * jref + 1))
    pj = np.zeros((ne, jtotmax + 1))
    for om in range(-jref, jref + 1):
        for ie in range(1, nel + 1):
            for iv in range(nv0, nv1 + 1):
                for j in range(nj):
                    for J in range(abs(om), jtotmax + 1):
                        if J < jc[-1]:
                            lo = [x for x in jc if x <= J]
                            if not lo:
                                raise ValueError("J = %d lies below the first calculated J, where the program "
                                                 "reads values it never set" % J)
                            j1 = lo[-1]
                            j2 = jc[jc.index(j1) + 1]
                            s1 = _column(tables, (om, j1, iv, ie), j, egrid, be[j1] * (J * (J + 1) - j1 * (j1 + 1)))
                            if J == j1:
                                s = s1
                            else:
                                s2 = _column(tables, (om, j2, iv, ie), j, egrid,
                                             be[j2] * (J * (J + 1) - j2 * (j2 + 1)))
                                s1 = np.where(np.isnan(s1), 0.0, s1)
                                s2 = np.where(np.isnan(s2), 0.0, s2)
                                s = ((j2 - J) * s1 + (J - j1) * s2) / float(j2 - j1)
                        else:
                            j1 = jc[-1]
                            s = _column(tables, (om, j1, iv, ie), j, egrid, be[j1] * (J * (J + 1) - j1 * (j1 + 1)))
                        s = np.where(s < 0.0, 0.0, s)
                        out[:, j, iv - nv0, ie - 1, om + jref] += s * (2 * J + 1)
                        pj[:, J] += s
    return out, pj


def k2(egrid_ev, xmasa):
    """k^2 = 2 mu E / hbar^2 with E in zot, the second column of the files (:400-404)."""
    ener = np.asarray(egrid_ev) / CEVCM * CONVE1
    return 2.0 * xmasa * ener / HBR / HBR


def write_files(outdir, egrid, xmasa, crpv, pj, nv0, jref):
    """CRPtot.res, CRPvib.res, CRPomg.res, PJ.res and CRP.vfVV.efE (:386-480)."""
    kk = k2(egrid, xmasa)
    ne, nj, nv, nel, nom = crpv.shape
    f15 = lambda vals: "".join(" %15.7E" % v for v in vals) + "\n"
    f16 = lambda vals: "".join(" %16.7E" % v for v in vals) + "\n"
    pj = np.where(pj < 1e-50, 0.0, pj)
    with open(os.path.join(outdir, "CRPtot.res"), "w") as ft, \
            open(os.path.join(outdir, "CRPvib.res"), "w") as fv, \
            open(os.path.join(outdir, "CRPomg.res"), "w") as fo, \
            open(os.path.join(outdir, "PJ.res"), "w") as fp:
        ft.write(" # Energy(eV)  k^2(Angstrom^2)  CRP \n")
        for i in range(ne):
            fp.write(f16((egrid[i],) + tuple(pj[i])))
            v = crpv[i].sum(axis=(0, 2, 3))
            v = np.where(v < 1e-30, 0.0, v)
            fv.write(f15((egrid[i], kk[i]) + tuple(v)))
            ft.write(f15((egrid[i], kk[i], crpv[i].sum())))
            fo.write(f15((egrid[i], kk[i]) + tuple(crpv[i].sum(axis=(0, 1, 2)))))
    for iv in range(nv):
        for ie in range(nel):
            with open(os.path.join(outdir, "CRP.vf%02d.ef%d" % (nv0 + iv, ie + 1)), "w") as f:
                for i in range(ne):
                    s = crpv[i, :, iv, ie, :].sum(axis=1)
                    s = np.where(s < 1e-60, 0.0, s)
                    f.write(f15((egrid[i], kk[i]) + tuple(s)))


def run_program(workdir, base=None):
    """The program: input.dat and CalculatedJ.dat in workdir, the tables under
    base (workdir/..), the result files into workdir.  Returns (E, CRP, PJ)."""
    from .host import namelist
    base = base or os.path.join(workdir, "..")
    g = namelist.read(os.path.join(workdir, "input.dat"))
    gb, pr, pm, fl, sg = g["inputgridbase"], g["inputprod"], g["inputpotmass"], g["inputflux"], g["sigmas2prod"]
    iprod = int(pr["iprod"])
    xm0, xm1, xm2 = float(pm["xm0"]), float(pm["xm1"]), float(pm["xm2"])
    xmtot = xm0 + xm1 + xm2
    if iprod == 1:
        j0, j1, nv0, nv1, nel = int(gb["jini"]), int(gb["jmax"]), int(gb["nvini"]), int(gb["nvmax"]), int(
            gb["nelecmax"])
        xmasa = xm1 * (xm0 + xm2) / xmtot
    elif iprod == 2:
        j0, j1, nv0, nv1, nel = int(pr["jiniprod"]), int(pr["jmaxprod"]), int(pr["nviniprod"]), int(
            pr["nvmaxprod"]), 1
        xmasa = xm2 * (xm0 + xm1) / xmtot
    else:
        raise ValueError("CRP needs product distributions (iprod = 1 or 2)")
    jref = int(gb["jref"])
    jc, be = read_calculated_j(os.path.join(workdir, "CalculatedJ.dat"), int(sg["ncalc"]))
    ne = int(sg["nesigma"])
    emin, emax = float(sg["eminsigma_ev"]), float(sg["emaxsigma_ev"])
    egrid = emin + np.arange(ne, dtype=np.float64) * ((emax - emin) / float(ne - 1))
    tables = read_tables(base, jc, jref, nv0, nv1, nel, int(fl["netot"]))
    crpv, pj = crp(tables, jc, be, int(sg["jtotmax"]), jref, egrid, nv0, nv1, nel, j1 - j0 + 1)
    write_files(workdir, egrid, xmasa, crpv, pj, nv0, jref)
    return egrid, crpv, pj
