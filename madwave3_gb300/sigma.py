"""Reaction cross sections from the per-J probability files, as the
post-processing program sigmaFromS2prod does
(SRC/AUXILIARy-CODES/sigmaFromS2prod.f): read P_J(E) (second column of each
J's S2prod, fourth for the product-resolved sum when iprod = 2), bring every
J from 0 to Jtotmax onto the cross-section energy grid by J-shifting
(JshiftInterPol, :317-478) and sum

    sigma(E) = pi / (k^2 (2 jref + 1)) sum_J (2J + 1) sum_Omega P_J^Omega(E),
    k^2 = 2 mu E (atomic units), reported in angstrom^2 (:255-272).

A calculated J is splined in energy; a J between two calculated ones is the
average of both, each shifted by B_J (J(J+1) - J_i(J_i+1)) and weighted by its
distance; a J above the last calculated one is the last one shifted.  Shifted
energies below a calculation's grid give 0, above it the last value.  The
spline is the reference's (SPLSET / SPLINQQ, restated in host/transcoor.py).
Energies of the grid: E_min + (i - 1) (E_max - E_min) / nESigma, i = 1..nESigma,
as the program does.
"""
import math

import numpy as np

from .host.transcoor import splinqq, splset

CONVL = 0.52917726          # bohr -> angstrom
CONVE = 4.55633538e-6       # cm^-1 -> hartree
CONVM = 0.182288853e4       # amu -> electron masses
CEVCM = 1.23984245e-4       # eV per cm^-1


def ev_to_au(e_ev):
    return e_ev * CONVE / CEVCM


def read_pj(path, iprod=0):
    """(E in hartree, P_J(E), P_J^prod(E)) of one S2prod file, P clipped at 1
    (sigmaFromS2prod.f:181-196)."""
    a = np.loadtxt(path, ndmin=2)
    e = ev_to_au(a[:, 0])
    p = np.minimum(a[:, 1], 1.0)
    pp = np.minimum(a[:, 3], 1.0) if iprod >= 2 else np.zeros_like(p)
    return e, p, pp


def _spline_at(e, p, x):
    d = splset(p, e)
    return np.array([splinqq(p, d, e, t) for t in x])


def _shifted(e, p, x, shift):
    d = splset(p, e)
    out = np.empty(len(x))
    for i, t in enumerate(x):
        s = t - shift
        if e[0] <= s <= e[-1]:
            out[i] = splinqq(p, d, e, s)
        elif s < e[0]:
            out[i] = 0.0
        else:
            out[i] = p[-1]
    return out


def jshift_pj(calc, be, jtotmax, egrid):
    """JshiftInterPol for one Omega: calc {J: (E, P)} of the calculated J
    (E in hartree), be {J: B_J in hartree}; returns PJ[len(egrid)][jtotmax + 1]."""
    js = sorted(calc)
    pj = np.zeros((len(egrid), jtotmax + 1))
    for J in range(jtotmax + 1):
        if J in calc:
            e, p = calc[J]
            pj[:, J] = _spline_at(e, p, egrid)
            continue
        lo = [j for j in js if j < J]
        hi = [j for j in js if j > J]
        if lo and hi:
            j0, j1 = lo[-1], hi[0]
            p0 = _shifted(*calc[j0], egrid, be[j0] * (J * (J + 1) - j0 * (j0 + 1)))
            p1 = _shifted(*calc[j1], egrid, be[j1] * (J * (J + 1) - j1 * (j1 + 1)))
            pj[:, J] = (j1 - J) / (j1 - j0) * p0 + (J - j0) / (j1 - j0) * p1
        elif J > js[-1]:
            j0 = js[-1]
            pj[:, J] = _shifted(*calc[j0], egrid, be[j0] * (J * (J + 1) - j0 * (j0 + 1)))
    return pj


def cross_section(pj_by_omega, egrid, xm0, xm1, xm2, iprod, jref=0):
    """sigma(E) in angstrom^2 (sigmaFromS2prod.f:117-130, 255-272).
    pj_by_omega {Omega: PJ[nE][J]}; masses in amu; iprod = 1 uses the product
    arrangement's reduced mass, otherwise the reactant's."""
    m0, m1, m2 = xm0 * CONVM, xm1 * CONVM, xm2 * CONVM
    mt = m0 + m1 + m2
    mu = m1 * (m0 + m2) / mt if iprod == 1 else m2 * (m0 + m1) / mt
    egrid = np.asarray(egrid, np.float64)
    k2 = 2.0 * mu * egrid
    fac = math.pi / (k2 * (2 * jref + 1)) * CONVL * CONVL
    tot = np.zeros(len(egrid))
    for om, pj in pj_by_omega.items():
        for J in range(pj.shape[1]):
            if abs(om) <= min(jref, J):
                tot += (2 * J + 1) * pj[:, J]
    return tot * fac


def energy_grid(emin_ev, emax_ev, nesigma):
    """The program's grid (dE = (Emax - Emin) / nESigma, nESigma points from Emin)."""
    emin, emax = ev_to_au(emin_ev), ev_to_au(emax_ev)
    return emin + np.arange(nesigma) * (emax - emin) / nesigma
