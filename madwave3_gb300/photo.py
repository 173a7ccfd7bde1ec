"""Photodissociation start (iphoto = 1, 2) on the host: the transition dipole
on the grid, the dipole-weighted bound state that becomes the initial packet,
its normalisation and the autocorrelation file (SRC/mod_photoini_01y2.f).

* ``threej``: the 3j symbol by Racah's formula, as ``tresj`` evaluates it with
  logarithms of factorials (SRC/liboctdyn.f:1154-1195, 215-230, 1443-1460).
* ``factresj``: dip_bnd's coefficients of the transition operator for
  linearly polarised light, parity-adapted (SRC/mod_photoini_01y2.f:236-270).
* ``dipole_table`` / ``write_dipole_files`` / ``read_dipole_files``:
  set_trans_dipole and read_trans_dipole (:32-190) for one bound electronic
  state: d_0 = d_z, d_{+-1} = -+ d_x / sqrt 2 (or d_{+-1} = d_y / sqrt 2 when
  only d_y is non-zero) at every stored point, from a ``dipele(r, R, cos)``
  callable (the reference's dipele_general.f interface, atomic units).
* ``initial_packet``: dip_bndgrid (:509-717) for iphoto = 1 (sum over the
  bound state's Omega and electronic states of bndvec x dipole x factresj)
  and 2 (the bound state itself), then dip_bnd's renormalisation (:330-380);
  the norm before it is photonorm, the scale of every printed probability.
* ``write_auto_file``: the autocorrelation file the spectra program reads
  (:384-415 and check, SRC/main_madwave3.f:444-455).
"""
import math
import os
from fractions import Fraction

import numpy as np

from .host.constants import conve1, convl, eV2cm


def _triangle(j1, j2, j3):
    """trian: sqrt((j1+j2-j3)! (j1-j2+j3)! (-j1+j2+j3)! / (j1+j2+j3+1)!), 0
    outside the triangle."""
    if j3 < abs(j1 - j2) or j3 > j1 + j2:
        return Fraction(0)
    f = math.factorial
    return Fraction(f(j1 + j2 - j3) * f(j1 - j2 + j3) * f(-j1 + j2 + j3), f(j1 + j2 + j3 + 1))


def threej(j1, j2, j3, m1, m2, m3):
    """(j1 j2 j3 / m1 m2 m3) for integer arguments, Racah's sum evaluated exactly."""
    if m1 + m2 + m3 != 0 or abs(m1) > j1 or abs(m2) > j2 or abs(m3) > j3:
        return 0.0
    tri = _triangle(j1, j2, j3)
    if tri == 0:
        return 0.0
    f = math.factorial
    k1, k2, k3, k4, k5 = j3 - j2 + m1, j3 - j1 - m2, j1 + j2 - j3, j1 - m1, j2 + m2
    s = Fraction(0)
    for k in range(max(-k1, -k2, 0), min(k3, k4, k5) + 1):
        term = Fraction(1, f(k) * f(k3 - k) * f(k4 - k) * f(k5 - k) * f(k1 + k) * f(k2 + k))
        s += -term if k % 2 else term
    pref = Fraction(f(j1 + m1) * f(j1 - m1) * f(j2 + m2) * f(j2 - m2) * f(j3 + m3) * f(j3 - m3))
    sign = -1 if (j1 - j2 - m3) % 2 else 1
    return sign * float(s) * math.sqrt(float(pref * tri))


def factresj(Jtot, iparity, Jtotini, iparini, max_omega=5):
    """dip_bnd's factresj(iomini, q, iom) as an array [iomini][q + 1][iom] over
    0..max(Jtot, Jtotini, max_omega); zero for transitions the parities forbid."""
    m = max(Jtot, Jtotini, max_omega)
    out = np.zeros((m + 1, 3, m + 1))
    for iom in range(max_omega + 1):
        for iomini in range(max_omega + 1):
            for iq in (-1, 0, 1):
                ssign = (-1.0) ** (iom + iq)
                yyy = 1.0
                if iom == 0:
                    yyy /= math.sqrt(2.0)
                if iomini == 0:
                    yyy /= math.sqrt(2.0)
                if iparity * iparini >= 0:
                    yyy = 0.0
                if iomini <= Jtotini and iom <= Jtot:
                    coef = threej(Jtotini, 1, Jtot, iomini, iq, -iom)
                    coef2 = threej(Jtotini, 1, Jtot, -iomini, iq, -iom)
                    xxx = coef + coef2 * float(iparini * (-1) ** Jtotini)
                    out[iomini, iq + 1, iom] = ssign * yyy * xxx
    return out


def _jacobi(run, iang, ir1, ir2):
    i = run.inp
    r1 = i.rmis1 + (ir1 - 1) * run.ah1
    r2 = i.rmis2 + (ir2 - 1) * run.ah2
    return r1 / convl, r2 / convl, float(run.cgamma[iang - 1])


def dipole_table(run, dipele):
    """set_trans_dipole for nelec_bnd = 1: dipol[nangu][npuntot][nelec][3] with the
    last index q + 1 (q = -1, 0, 1); dipele(rpeq, Rg, cos gamma) returns the
    (dx, dy, dz) arrays of the nelec final states."""
    i = run.inp
    ne = run.nelec
    out = np.zeros((i.nangu, run.npuntot, ne, 3))
    s2 = math.sqrt(2.0)
    for iang in range(1, i.nangu + 1):
        for ir in range(run.npunreal[iang - 1]):
            rpeq, rg, cg = _jacobi(run, iang, int(run.indr1[iang - 1, ir]), int(run.indr2[iang - 1, ir]))
            dx, dy, dz = (np.broadcast_to(np.asarray(v, np.float64), (ne,)) for v in dipele(rpeq, rg, cg))
            for e in range(ne):
                if abs(dx[e]) > 1e-10 or abs(dz[e]) > 1e-10:
                    out[iang - 1, ir, e] = (dx[e] / s2, dz[e], -dx[e] / s2)
                elif abs(dy[e]) > 1e-10:
                    out[iang - 1, ir, e] = (dy[e] / s2, 0.0, dy[e] / s2)
    return out


def write_dipole_files(outdir, run, dipol):
    """dip/dip.NNN.dat rows 'ir1 ir2 (dip(q, ielec), ielec), q = -1..1' (nelec_bnd = 1)."""
    os.makedirs(os.path.join(outdir, "dip"), exist_ok=True)
    for iang in range(1, run.inp.nangu + 1):
        with open(os.path.join(outdir, "dip", "dip.%03d.dat" % iang), "w") as f:
            for ir in range(run.npunreal[iang - 1]):
                vals = [dipol[iang - 1, ir, e, q] for q in range(3) for e in range(run.nelec)]
                f.write("%d %d %s\n" % (run.indr1[iang - 1, ir], run.indr2[iang - 1, ir],
                                        " ".join(repr(float(v)) for v in vals)))


def read_dipole_files(outdir, run):
    """read_trans_dipole: the table back from dip/ (nelec_bnd = 1)."""
    ne = run.nelec
    out = np.zeros((run.inp.nangu, run.npuntot, ne, 3))
    for iang in range(1, run.inp.nangu + 1):
        n = run.npunreal[iang - 1]
        d = np.loadtxt(os.path.join(outdir, "dip", "dip.%03d.dat" % iang), ndmin=2)[:n]
        out[iang - 1, :n] = d[:, 2:].reshape(n, 3, ne).transpose(0, 2, 1)
    return out


def initial_packet(run, bnddir, iv, iphoto, Jtotini=None, iparini=None, dipol=None, nelec_bnd=1, idproc=0):
    """dip_bndgrid + dip_bnd's normalisation.  The bound state is read from the
    bnd.ivNNN / grid files write_bnd stored (the same grid).  Returns
    (psi0 normalised, photonorm = its norm before, energy of the bound state
    in eV, {Omega: probability})."""
    from .bndlanz import _point_labels, read_bound_state
    key, (nr1, nr2, nang, omax, nel), e_ev = read_bound_state(run, bnddir, iv, idproc)
    me = _point_labels(run)
    psi0 = np.zeros(run.ntot)
    if iphoto == 1:
        if dipol is None or Jtotini is None or iparini is None:
            raise ValueError("iphoto = 1 needs the dipole table and Jtotini, iparini")
        fr = factresj(run.inp.Jtot, run.inp.iparity, Jtotini, iparini)
        if not np.any(np.abs(fr) > 1e-10):
            raise ValueError("forbidden transition for iphoto = 1: check the rotational quantum numbers")
    for k in range(run.ntot):
        icanp, ielec, iom, iangp, ir, ir1, ir2, iang = (int(x) for x in me[k])
        if not (ir1 <= nr1 and ir2 <= nr2 and iang <= nang):
            continue
        if iphoto == 2:
            if iom <= omax and ielec <= nelec_bnd:
                psi0[k] += key.get((ir1, ir2, iang, iom, ielec), 0.0)
        else:
            for eb in range(1, nelec_bnd + 1):
                for iomini in range(0, omax + 1):
                    iq = iom - iomini
                    if abs(iq) <= 1:
                        y = dipol[iang - 1, ir - 1, ielec - 1, iq + 1]
                        x = fr[iomini, iq + 1, iom]
                        psi0[k] += key.get((ir1, ir2, iang, iomini, eb), 0.0) * y * x
    xnorm = float(np.dot(psi0, psi0))
    if xnorm < 1e-15:
        raise ValueError("norm of the initial packet too low: %g" % xnorm)
    per_om = {}
    for k in range(run.ntot):
        om = int(me[k][2])
        per_om[om] = per_om.get(om, 0.0) + psi0[k] * psi0[k] / xnorm
    return psi0 / math.sqrt(xnorm), xnorm, e_ev, per_om


def fortran_d(x, w=20, d=12):
    """Fortran Dw.d (0.ddd...D+ee, leading blank when the field allows)."""
    if x == 0.0:
        body = "0." + "0" * d + "D+00"
    else:
        e = int(math.floor(math.log10(abs(x)))) + 1
        m = abs(x) / 10.0 ** e
        mr = round(m, d)
        if mr >= 1.0:
            mr /= 10.0
            e += 1
        body = ("%." + str(d) + "f") % mr
        body = body[1:] if body.startswith("0") else body
        body = "0" + body if not body.startswith("0") else body
        body += "D%+03d" % e
        if x < 0:
            body = "-" + body
    return body.rjust(w)


def write_auto_file(path, photonorm, energy_ini_ev, emindlt, delta2, iterations, autos):
    """auto.vVV.jJJ.JJJJ: the header (4(1x,d20.12)) photonorm, the bound state's
    energy, emindlt and delta2, then 'k <psi0|psi_k>' per iteration."""
    with open(path, "w") as f:
        f.write("".join(" " + fortran_d(v) for v in (photonorm, energy_ini_ev, emindlt, delta2)) + "\n")
        for k, a in zip(iterations, autos):
            f.write(" %12d %r\n" % (int(k), float(a)))


def auto_file_name(run):
    i = run.inp
    return "auto.v%02d.j%02d.J%03d" % (i.nvref, i.jref, i.Jtot)


def bound_energy_zot(e_ev):
    return e_ev * eV2cm * conve1
