"""The per-loop probability files of the time loop (printprob,
SRC/main_madwave3.f:555-844) from the library's accumulators, in the
reference's formats, so the post-processing programs of
SRC/AUXILIARy-CODES (sigmaFromS2prod, CRP-fast, ...) read them unchanged.

Written for a diatom (xm2 > 1e-3) and iprod = 0, 1 or 2; every probability
is multiplied by photonorm, 1 for collisions (mod_flux_01y2.f:416) and the
norm |d.e psi|^2 of the initial packet for photodissociation (dip_bnd,
SRC/mod_photoini_01y2.f:384-386):

* ``S2prod.vVV.JJJJ.kKKKKK``, one line per energy, format (501(1x,e17.7e3)):
  iprod = 0: E (eV), P(E) (S2prodtot), P(E) + S2reac, reacfct(E)
  (main_madwave3.f:712-716); iprod = 1: E, S2reac, P(E) + S2reac, then the
  vibrational distribution of every electronic state (:719-725); iprod = 2
  (product projection, one product electronic state or diabatic products,
  :734-741): E, P(E), P(E) + S2reac, S2no, the product v' distribution, from
  zS2prod with S2pro(v,j,Omega) = |zS2prod|^2 / (4 pi^2) S2prodfac(E,v,j)
  (:669-684).
* ``S2prodelec``: E and the per-electronic-state P(E) (:717-718, :726-727).

S2reac(E) is the sum over the reactant-channel elements
S2(v,j,block) = |zS2(E,v,j,block) / 2 pi|^2 S2factor(E,v,j,e) for j = j00(block)
..jmax step inc and v = nvini..noBCstates(j,e) (:640-652).  Values below 1e-90
are written as 0 (:700-705).  The diatom-only case and the adiabatic
product assignment of iprod = 2 with several product states (vibelecprod)
are not written here.
"""
import os

import numpy as np

from .host.constants import conve1, eV2cm, pi


def fortran_e(x, w, d, ex_digits=2):
    """Fortran Ew.d (ex_digits = 2) or Ew.dEe (ex_digits = e) output of x: a
    0.ddd mantissa of d digits rounded to nearest, right-aligned in w."""
    x = float(x)
    if x == 0.0:
        s = "0." + "0" * d + "E+" + "0" * ex_digits
    else:
        m, e = ("%.*E" % (d - 1, abs(x))).split("E")     # d significant digits
        ex = int(e) + 1
        s = "0." + m.replace(".", "") + "E" + ("+" if ex >= 0 else "-") + "%0*d" % (ex_digits, abs(ex))
        if x < 0:
            s = "-" + s
    return "%*s" % (w, s)


def e17_7e3(x):
    """Fortran E17.7E3, the format of every S2prod column."""
    return fortran_e(x, 17, 7, 3)


def _line(vals):
    return "".join(" " + e17_7e3(v) for v in vals) + "\n"


def s2_elements(run, zs2, s2factor):
    """S2(ie, v, j, block) of every reactant-channel element that printprob sums
    (main_madwave3.f:640-652); zs2 [ncan][nj][nv][netot] complex, s2factor
    [nelec][nj][nv][netot].  Returns S2 [ncan][nj][nv][netot] (0 off the sum)."""
    i = run.inp
    out = np.zeros(zs2.shape, np.float64)
    for b in range(run.ncan):
        e = int(run.nelebas[b]) - 1
        for j in range(int(run.j00[b]), i.jmax + 1, i.inc):
            jj = j - i.jini
            nob = int(run.nobc[e, jj])
            for iv in range(i.nvini, nob + 1):
                vv = iv - i.nvini
                z = zs2[b, jj, vv] / 2.0 / pi
                out[b, jj, vv] = (z.real * z.real + z.imag * z.imag) * s2factor[e, jj, vv]
    return out


def s2prod_products(zs2prod, s2prodfac, pp):
    """S2pro summed over Omega and j into (S2no(E), vibprod(v', E)) for iprod = 2
    (main_madwave3.f:669-684).  zs2prod [nom][njp][nvp][netot] complex (the
    library's mw3_download_product), s2prodfac [njp][nvp][netot]."""
    z = np.asarray(zs2prod)
    a = (z.real * z.real + z.imag * z.imag) * 0.25 / (pi * pi) * np.asarray(s2prodfac)[None]
    nom, njp, nvp = pp.shape
    mask = np.zeros((njp, nvp), bool)
    for jj in range(njp):
        mask[jj, : int(pp.nobcprod[jj]) - pp.nviniprod + 1] = True
    a = a * mask[None, :, :, None]
    return a.sum(axis=(0, 1, 2)), a.sum(axis=(0, 1))


def write_s2prod(outdir, run, iloop, s2prodtot, s2prodelec, zs2, etot, reacfct, s2factor, nvmaxprod=None,
                 iprod=None, product=None, photonorm=1.0):
    """Writes S2prod.vVV.JJJJ.kKKKKK and S2prodelec for one loop; returns the
    S2prod path.  Arguments as the library returns them (``Propagator.totalflux``,
    ``.accumulators()['zs2']``, ``.tables()``); iprod defaults to the run's,
    and iprod = 2 takes product = (zs2prod, s2prodfac, ProductProjection).
    photonorm scales every probability (1 for collisions; |d.e psi|^2 of
    the photodissociation start, madwave3_gb300.photo.initial_packet)."""
    i = run.inp
    iprod = run.inp.iprod if iprod is None else iprod
    if iprod not in (0, 1, 2):
        raise ValueError("printprob is written for iprod = 0, 1 or 2")
    s2 = s2_elements(run, np.asarray(zs2), np.asarray(s2factor))
    s2reac = s2.sum(axis=(0, 1, 2))
    nelec = run.nelec
    vib = None
    if iprod == 2:
        if product is None:
            raise ValueError("iprod = 2 needs product = (zs2prod, s2prodfac, projection)")
        s2no, vib = s2prod_products(*product)
        s2no = np.where(s2no < 1e-90, 0.0, s2no)
        vib = np.where(vib < 1e-90, 0.0, vib)
    if iprod == 1:
        if nvmaxprod is None:
            raise ValueError("iprod = 1 needs nvmaxprod (&inputprod)")
        vtop = min(nvmaxprod, i.nvmax)
        vib = np.zeros((nelec, vtop - i.nvini + 1, len(etot)))
        for b in range(run.ncan):
            e = int(run.nelebas[b]) - 1
            for j in range(int(run.j00[b]), i.jmax + 1, i.inc):
                jj = j - i.jini
                for iv in range(i.nvini, min(nvmaxprod, int(run.nobc[e, jj])) + 1):
                    vib[e, iv - i.nvini] += s2[b, jj, iv - i.nvini]
        vib[vib < 1e-90] = 0.0
    tot = np.where(np.asarray(s2prodtot) < 1e-90, 0.0, s2prodtot)
    s2reac = np.where(s2reac < 1e-90, 0.0, s2reac)
    pn = float(photonorm)
    if pn != 1.0:
        tot, s2reac = tot * pn, s2reac * pn
        s2prodelec = [np.asarray(x) * pn for x in s2prodelec]
        if vib is not None:
            vib = vib * pn
        if iprod == 2:
            s2no = s2no * pn
    name = os.path.join(outdir, "S2prod.v%02d.J%03d.k%05d" % (i.nvref, i.Jtot, iloop))
    e_ev = np.asarray(etot) / conve1 / eV2cm
    with open(name, "w") as f, open(os.path.join(outdir, "S2prodelec"), "w") as fe:
        for ie in range(len(etot)):
            if iprod == 0:
                f.write(_line([e_ev[ie], tot[ie], tot[ie] + s2reac[ie], reacfct[ie]]))
            elif iprod == 2:
                f.write(_line([e_ev[ie], tot[ie], tot[ie] + s2reac[ie], s2no[ie]] + list(vib[:, ie])))
            else:
                f.write(_line([e_ev[ie], s2reac[ie], tot[ie] + s2reac[ie]] + list(vib[:, :, ie].ravel())))
            fe.write(_line([e_ev[ie]] + [s2prodelec[e][ie] for e in range(nelec)]))
    return name


def read_s2prod(path):
    """The columns of an S2prod file as the post-processing programs read them
    (list-directed: sigmaFromS2prod takes E and P_J(E) from the first two,
    AUXILIARy-CODES/sigmaFromS2prod.f:181-189)."""
    return np.loadtxt(path, ndmin=2)
