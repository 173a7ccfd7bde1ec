"""State-to-state product distributions from the per-iteration Cvjprod
records, as the post-processing program distriwvp does for product-state
projections (SRC/AUXILIARy-CODES/distriwvp.f, the iprod = 2 branch).

The propagation writes, per block of ntimes iterations, Cvjprod.NNNN: one
unformatted record 'it, Cvjprod(nviniprod:nvmaxprod, jiniprod:jmaxprod,
iomminprod:iommaxprod)' per iteration (madwave3_gb300.contfiles).  The
program reads the records of Cvjprod.0001 .. .nloop in order (stopping at the
first missing file; a file with fewer than ntimes records is an error) and,
with k the record's position, rebuilds on the translational-energy grid
E = Ekin_min + (ie - 1) (Ekin_max - Ekin_min) / (netot - 1)

    zS2prod(v, j, Omega; E) = sum_k (2 hbar / delta2) exp(-i k acos Es) / sqrt(1 - Es^2) Cvjprod_k(v, j, Omega),
    Es = (E - emindlt) / delta2,

the sum the propagation accumulates (:457-481), with emindlt and delta2 from
pot/cont.pot and the input's cut-offs (:121-147) and hbar its own literal
0.063533625.  The propagation numbers its iterations from 2 on a fresh start
(SRC/main_madwave3.f:250, :324) and adds Cvjprod_it C_it(E), so with k the
record's position every term is the accumulator's times exp(i acos Es): the
program's zS2prod is the accumulator times that phase, and |zS2prod|^2, all it
writes, is the same.  Then S2 = |zS2prod / 2 pi|^2 S2prodfac, with S2prodfac =
hbar^2 pfin pini / (2 paqini mu mu') for collisions (paqini: the packet's
energy distribution on a 1024-point R grid, pini = sqrt(2 mu E)/hbar,
pfin = sqrt(2 mu' (E - E'(v, j) + E_ref))/hbar, zero unless paqini > 1e-10
and E > Emincut_prod; :390-441) or 4 pfin / (pi mu') for photodissociation,
and the files distriS2prod.vVV.e1 (E, then for each j the sum over Omega of
S2) and distriS2prod.vib (E, the total, then each v's sum), all times
photonorm (:487-525).  Product energies E'(v, j) come from func/prodwf as
stored, E_ref = E(nvref, jref, ielecref) from func/bcwf.
"""
import math
import os

import numpy as np

from .contfiles import read_cvj_file

# distriwvp.f:56-66
CONVE1 = 1.197e-4
HBR = 0.063533625
EV2CM = 8065.5
NPUNT = 1024


def energy_interval(vmin, vmaxtot, radcutmax_ev, rotcutmax_ev):
    """emindlt, delta2 from cont.pot's vmin and vmaxtot (zot) and the input's
    radial and rotational cut-offs (distriwvp.f:139-147)."""
    vmaxtot_ev = vmaxtot / (EV2CM * CONVE1)
    emaxtot = (vmaxtot_ev + radcutmax_ev + 3.0 * rotcutmax_ev) * EV2CM * CONVE1
    delta2 = 0.5 * (emaxtot - vmin)
    return vmin + delta2, delta2


def energy_grid(ekinmin_ev, ekinmax_ev, netot):
    """The translational energies (zot) of the distributions (:390-394)."""
    emin, emax = ekinmin_ev * EV2CM * CONVE1, ekinmax_ev * EV2CM * CONVE1
    return emin + np.arange(netot, dtype=np.float64) * ((emax - emin) / float(netot - 1))


def read_records(directory, nloop, ntimes, shape, prefix="Cvjprod"):
    """The Cvjprod arrays of iterations 1.. in order (:282-307), as [K][shape]."""
    rows = []
    for iloop in range(1, nloop + 1):
        path = os.path.join(directory, "%s.%04d" % (prefix, iloop))
        if not os.path.exists(path):
            break
        _, r = read_cvj_file(path, shape)
        if len(r) < ntimes:
            raise ValueError("%s for iloop=%d not complete, ik=%d" % (prefix, iloop, len(r) + 1))
        rows.extend(r[:ntimes])
    return np.array(rows)


def chebyshev_sum(records, energies, emindlt, delta2, hbr=HBR):
    """zS2prod[..., ie]: the records' damped-free Chebyshev transform (:457-481),
    k = 1 for the first record."""
    records = np.asarray(records, dtype=np.float64)
    kk = np.arange(1, records.shape[0] + 1, dtype=np.float64)
    es = (np.asarray(energies) - emindlt) / delta2
    with np.errstate(invalid="ignore"):
        c = (2.0 * hbr / delta2) * np.exp(-1j * np.outer(kk, np.arccos(es))) / np.sqrt(1.0 - es * es)
    flat = records.reshape(records.shape[0], -1)
    return (flat.T @ c).reshape(records.shape[1:] + (len(es),))


def _riccati(l, x):
    """F = x j_l(x), G = x y_l(x), the open-channel BESPH2 solutions (G ~ -cos(x - l pi / 2))."""
    from scipy.special import spherical_jn, spherical_yn
    return x * spherical_jn(l, x), x * spherical_yn(l, x)


def packet_distribution(energies, rmis2, rfin2, rcolini, ecol_ev, deltae_ev, xmasa, Jtot, jref, iomref, hbr=HBR,
                        npunt=NPUNT):
    """(paqini, pini) per energy: the collision packet's projection on the
    outgoing Riccati-Bessel waves of its l (:333-415), on npunt R points (the
    program's 1024; the propagation's Smatini_col takes 1000)."""
    ecol = ecol_ev * EV2CM * CONVE1
    deltae = deltae_ev * EV2CM * CONVE1
    xk0 = math.sqrt(2.0 * xmasa * ecol) / hbr
    alpha0 = math.sqrt(2.0 * ecol / xmasa) * hbr / deltae
    factor = (2.0 / math.pi / alpha0 / alpha0) ** 0.25
    ah = (rfin2 - rmis2) / float(npunt - 1)
    det = float(Jtot * (Jtot + 1) + jref * (jref + 1) - 2 * iomref * iomref)
    il = int(0.5 * (-1.0 + math.sqrt(1.0 + 4.0 * det)) + 0.5)
    r = rmis2 + np.arange(npunt, dtype=np.float64) * ah
    zg = np.cos((r - rcolini) * xk0) * math.sqrt(2.0) * factor * np.exp(-(r - rcolini) ** 2 / alpha0 ** 2)
    zg = zg / math.sqrt(2.0)
    paq, pini = np.zeros(len(energies)), np.zeros(len(energies))
    for ie, e in enumerate(energies):
        if e <= 0.0:
            continue
        p = math.sqrt(e * xmasa * 2.0 / hbr / hbr)
        f, g = _riccati(il, r * p)
        keep = np.abs(f) > 1e-20
        z = np.sum(zg[keep] * (-g[keep] + 1j * f[keep])) * ah / 2.0 / math.pi
        paq[ie] = (z * z.conjugate()).real
        pini[ie] = p
    return paq, pini


def s2prodfac(energies, ediatprod, ediatref, xmasaprod, paqini=None, pini=None, xmasa=None, emincut=0.0,
              iphoto=0, hbr=HBR):
    """S2prodfac[ie][v][j] (:417-441); ediatprod [v][j] in zot."""
    e = np.asarray(energies)[:, None, None]
    ekf = e - np.asarray(ediatprod)[None] + ediatref
    pfin = np.where(ekf > 0.0, np.sqrt(np.maximum(ekf, 0.0) * xmasaprod * 2.0 / hbr / hbr), 0.0)
    if iphoto > 0:
        return 4.0 * pfin / (math.pi * xmasaprod)
    paq = np.asarray(paqini)[:, None, None]
    pin = np.asarray(pini)[:, None, None]
    ok = (paq > 1e-10) & (e > emincut)
    with np.errstate(divide="ignore", invalid="ignore"):
        fac = hbr * hbr * pfin * pin / (2.0 * paq) / xmasa / xmasaprod
    return np.where(ok, fac, 0.0)


def distributions(zs2, fac, jiniprod, iomminprod, photonorm=1.0):
    """From zS2prod[nom][nj][nv][ne] and S2prodfac[ne][nv][nj]: the per-v tables
    vibrot[nv][ne][nj] (sum over Omega, j >= |Omega|), vibprod[nv][ne] and the
    total S2no[ne], all times photonorm (:487-525)."""
    nom, nj, nv, ne = zs2.shape
    s2 = np.abs(zs2 / 2.0 / math.pi) ** 2 * np.transpose(fac, (2, 1, 0))[None]      # [nom][nj][nv][ne]
    jv = jiniprod + np.arange(nj)
    om = iomminprod + np.arange(nom)
    mask = (jv[None, :] >= np.abs(om)[:, None]).astype(np.float64)                  # [nom][nj]
    s2 = s2 * mask[:, :, None, None]
    vibrot = np.transpose(s2.sum(axis=0), (1, 2, 0)) * photonorm                     # [nv][ne][nj]
    vibprod = vibrot.sum(axis=2)
    return vibrot, vibprod, vibprod.sum(axis=0)


def write_files(outdir, energies, vibrot, vibprod, s2no, nviniprod):
    """distriS2prod.vVV.e1 and distriS2prod.vib ('(1000(1x,e15.7))' lines)."""
    e_ev = np.asarray(energies) / (CONVE1 * EV2CM)
    fmt = lambda vals: "".join(" %15.7E" % v for v in vals) + "\n"
    for k in range(vibrot.shape[0]):
        with open(os.path.join(outdir, "distriS2prod.v%02d.e1" % (nviniprod + k)), "w") as f:
            for ie in range(len(e_ev)):
                f.write(fmt((e_ev[ie],) + tuple(vibrot[k, ie])))
    with open(os.path.join(outdir, "distriS2prod.vib"), "w") as f:
        for ie in range(len(e_ev)):
            f.write(fmt((e_ev[ie], s2no[ie]) + tuple(vibprod[:, ie])))


def run_program(rundir, potdir=None, funcdir=None, outdir=None):
    """The program for a product-state-projection run (iprod = 2): reads
    input.dat, the Cvjprod files and (photodissociation) the auto file in
    rundir, pot/cont.pot and func/bcwf, func/prodwf from ../ (potdir,
    funcdir), and writes the distriS2prod files into outdir (rundir).
    Returns (energies, vibrot, vibprod, S2no)."""
    from .host import namelist
    potdir = potdir or os.path.join(rundir, "..", "pot")
    funcdir = funcdir or os.path.join(rundir, "..", "func")
    outdir = outdir or rundir
    g = namelist.read(os.path.join(rundir, "input.dat"))
    gb, pr, pm = g["inputgridbase"], g["inputprod"], g["inputpotmass"]
    if int(pr.get("iprod", 0)) != 2:
        raise NotImplementedError("distributions are restated for product-state projections (iprod = 2)")
    iphoto = int(g.get("inputprocess", {}).get("iphoto", 0))
    tm, fl, co = g["inputtime"], g["inputflux"], g.get("inputcol", {})
    nv0, nv1 = int(pr["nviniprod"]), int(pr["nvmaxprod"])
    j0, j1 = int(pr["jiniprod"]), int(pr["jmaxprod"])
    om0, om1 = int(pr["iomminprod"]), int(pr["iommaxprod"])
    # cont.pot: nelec, one line per state, then vmin, maxpoint, vmaxtot (:121-138)
    with open(os.path.join(potdir, "cont.pot")) as f:
        lines = f.read().splitlines()
    nelec = int(lines[0].split()[0])
    t = [float(x.replace("D", "E")) for x in lines[1 + nelec].split()]
    vmin, vmaxtot = t[0], (t[2] if len(t) > 2 else float(pm["vcutmaxev"]))
    emindlt, delta2 = energy_interval(vmin, vmaxtot, float(pm["radcutmaxev"]), float(pm["rotcutmaxev"]))
    # E_ref from func/bcwf (:221-233), product energies from func/prodwf (:234-245), as stored
    from .host.setup import product_radialf_read
    ediatref = _bcwf_energy(os.path.join(funcdir, "bcwf"), int(gb["npun1"]), int(gb["jini"]), int(gb["nvini"]),
                            int(gb["nvref"]), int(gb["jref"]), int(gb["ielecref"]))
    _, ediatprod, _, _, _ = product_radialf_read(os.path.join(funcdir, "prodwf"), j0, j1, nv0, nv1,
                                                 int(pr["n2prod1"]))
    xm0, xm1, xm2 = float(pm["xm0"]), float(pm["xm1"]), float(pm["xm2"])
    xmtot = xm0 + xm1 + xm2
    xmasa, xmasaprod = xm2 * (xm0 + xm1) / xmtot, xm1 * (xm0 + xm2) / xmtot
    e = energy_grid(float(fl["ekinmin_ev"]), float(fl["ekinmax_ev"]), int(fl["netot"]))
    rec = read_records(rundir, int(tm["nloop"]), int(tm["ntimes"]), (om1 - om0 + 1, j1 - j0 + 1, nv1 - nv0 + 1))
    zs2 = chebyshev_sum(rec, e, emindlt, delta2)
    photonorm = 1.0
    emincut = float(pr.get("emincut_prod_ev", 0.0)) * EV2CM * CONVE1
    if iphoto > 0:
        name = "auto.v%02d.j%02d.J%03d" % (int(gb["nvref"]), int(gb["jref"]), int(gb["jtot"]))
        with open(os.path.join(rundir, name)) as f:
            photonorm = float(f.readline().split()[0].replace("D", "E"))
        fac = s2prodfac(e, ediatprod.T, ediatref, xmasaprod, iphoto=iphoto)
    else:
        paq, pini = packet_distribution(e, float(gb["rmis2"]), float(gb["rfin2"]), float(co["rcolini_ang"]),
                                        float(co["ecol_ev"]), float(co["deltae_ev"]), xmasa, int(gb["jtot"]),
                                        int(gb["jref"]), int(gb["iomref"]))
        fac = s2prodfac(e, ediatprod.T, ediatref, xmasaprod, paq, pini, xmasa, emincut)
    vibrot, vibprod, s2no = distributions(zs2, fac, j0, om0, photonorm)
    write_files(outdir, e, vibrot, vibprod, s2no, nv0)
    return e, vibrot, vibprod, s2no


def _bcwf_energy(path, npun1, jini, nvini, nvref, jref, ielecref):
    """E(nvref, jref, ielecref) of func/bcwf as stored (state blocks 'ielec j
    noBCstates', then per v 'v E' and npun1 values)."""
    with open(path) as f:
        toks = f.read().split()
    p = 0
    while p < len(toks):
        ie, j, nob = int(toks[p]), int(toks[p + 1]), int(toks[p + 2])
        p += 3
        for iv in range(nvini, nob + 1):
            if ie == ielecref and j == jref and iv == nvref:
                return float(toks[p + 1].replace("D", "E"))
            p += 2 + npun1
    raise ValueError("func/bcwf has no level v=%d j=%d of state %d" % (nvref, jref, ielecref))
