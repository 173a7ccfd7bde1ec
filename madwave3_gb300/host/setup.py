"""Host-side set-up of one madwave3 run (the modules the Fortran host keeps).

The GPU path replaces mod_Hphi_01y2, mod_absorcion_01y2, mod_flux_01y2 and
mod_PsiE_01y2.  Everything they consume is produced on the host by the
modules that stay: grid and Gauss-Legendre angles (mod_gridYpara_01y2),
masses/cut-offs and the compressed potential grid (mod_pot_01y2: pot0, pot2),
the Omega/electronic basis and Wigner functions (mod_baseYfunciones_01y2:
basis, paralelizacion for one process, angular_functions,
radial_functions01_read) and the initial collision packet (mod_colini_01y2).
This module restates those for a single process so that a run can be driven
without the Fortran program; :class:`Run` holds the arrays exactly in the
layout the C-ABI (``include/mw3gpu.h``) takes.

State vectors follow the reference's flat index ``indtotproc`` for nproc = 1
(SRC/mod_pot_01y2.f:435-455): angle-major with angles in the order
``indangreal`` gives them (nangu, nangu-1, ..., 1; SRC/mod_baseYfunciones_01y2.f:369-373),
then Omega/electronic block, then stored point.
"""
import math
import os
from dataclasses import dataclass

import numpy as np

from . import constants as C
from . import namelist
from .wigner import dwigner_vec, gauleg


def _get(d, key, default):
    return d.get(key.lower(), default)


@dataclass
class Inputs:
    """The namelist values of ``input.dat`` that the path depends on."""
    # &inputgridbase
    npun1: int = 0
    rmis1: float = 0.0
    rfin1: float = 0.0
    npun1min: int = 32
    npun2: int = 0
    rmis2: float = 0.0
    rfin2: float = 0.0
    nangu: int = 0
    Jtot: int = 0
    iparity: int = 1
    inc: int = 1
    nelecmax: int = 1
    iommin: int = 0
    iommax: int = 0
    j0: int = 0
    jini: int = 0
    jmax: int = 0
    nvini: int = 0
    nvmax: int = 0
    nvref: int = 0
    jref: int = 0
    iomref: int = 0
    ielecref: int = 1
    # &inputprod / &inputprocess
    iprod: int = 0
    iphoto: int = 0
    # &inputpotmass
    xm0: float = 0.0
    xm1: float = 0.0
    xm2: float = 0.0
    vcutmaxev: float = 0.0
    radcutmaxev: float = 0.0
    rotcutmaxev: float = 0.0
    radau: int = 0
    proj_j2_up: int = 0
    no_ref_energy: int = 1
    # &inputabsorcion
    absr1: float = 0.0
    absalp1: float = 0.0
    n1expo: int = 2
    ninterv1: int = 1
    absr2: float = 0.0
    absalp2: float = 0.0
    n2expo: int = 2
    ninterv2: int = 1
    # &inputcol
    rcolini_ang: float = 0.0
    ecol_ev: float = 0.0
    deltae_ev: float = 0.0
    # &inputflux
    r1flux_ang: float = 0.0
    netot: int = 0
    ekinmin_ev: float = 0.0
    ekinmax_ev: float = 0.0
    # &inputtime
    ntimes: int = 0
    nloop: int = 0
    kminelastic: int = 0

    @classmethod
    def from_namelists(cls, groups):
        self = cls()
        flat = {}
        for g in groups.values():
            flat.update(g)
        for f in self.__dataclass_fields__:
            key = f.lower()
            if key in flat:
                cur = getattr(self, f)
                v = flat[key]
                setattr(self, f, type(cur)(v) if not isinstance(cur, str) else v)
        return self

    @classmethod
    def read(cls, path):
        return cls.from_namelists(namelist.read(path))


@dataclass
class Run:
    """All host tables of one partial wave, in C-ABI layout (see module doc)."""
    inp: Inputs
    # grid (mod_gridYpara)
    ah1: float = 0.0
    ah2: float = 0.0
    nangu2: int = 0
    cgamma: np.ndarray = None
    wreal: np.ndarray = None
    # pot0
    xm1red: float = 0.0
    xm2red: float = 0.0
    xm1reac: float = 0.0
    xm2reac: float = 0.0
    xm1prod: float = 0.0
    xm2prod: float = 0.0
    vcutmax: float = 0.0
    radcutmax: float = 0.0
    rotcutmax: float = 0.0
    # cont.pot / pot2
    nelec: int = 1
    iomdiat: np.ndarray = None
    iomatom: np.ndarray = None
    sigdiat: np.ndarray = None
    sigatom: np.ndarray = None
    vmintot: float = 0.0
    vmaxtot: float = 0.0
    emindlt: float = 0.0
    delta2: float = 0.0
    npunreal: np.ndarray = None     # [nangu]
    npuntot: int = 0
    indr1: np.ndarray = None        # [nangu, npuntot] 1-based
    indr2: np.ndarray = None
    vvv: np.ndarray = None          # [nelec(je), nelec(ie), nangu, npuntot]
    # basis
    ncan: int = 0
    iombas: np.ndarray = None
    nelebas: np.ndarray = None      # 1-based electronic state
    j00: np.ndarray = None
    nojbas: np.ndarray = None
    jbas: np.ndarray = None         # [ncan, nangu]
    djmmp: np.ndarray = None        # [Jtot+1, nelec, nangu2+1, nangu]
    # radial functions (bcwf)
    nobc: np.ndarray = None         # [nelec, jmax-jini+1]
    ediat: np.ndarray = None        # [nelec, nj, nv]
    fd: np.ndarray = None           # [nelec, nj, nv, npun1]
    ediatref: float = 0.0
    # flat layout
    ntot: int = 0
    offs: np.ndarray = None         # [nangu, ncan] start of (iang, block) run
    psi0: np.ndarray = None
    # colini
    xmasa0: float = 0.0
    xk0: float = 0.0
    alpha0: float = 0.0
    factor0: float = 0.0
    il0: int = 0
    rcolini: float = 0.0
    gauss_norm: float = 0.0

    # ---- helpers -------------------------------------------------------
    def angle_order(self):
        """Angles (1-based) in flat-vector order: indangreal(:,0)."""
        return list(range(self.inp.nangu, 0, -1))

    def point_table(self):
        """Per flat index: (block 0-based, iang 1-based, ir1, ir2) arrays."""
        blk = np.empty(self.ntot, np.int32)
        ang = np.empty(self.ntot, np.int32)
        r1 = np.empty(self.ntot, np.int32)
        r2 = np.empty(self.ntot, np.int32)
        for iang in self.angle_order():
            n = self.npunreal[iang - 1]
            for b in range(self.ncan):
                o = self.offs[iang - 1, b]
                blk[o:o + n] = b
                ang[o:o + n] = iang
                r1[o:o + n] = self.indr1[iang - 1, :n]
                r2[o:o + n] = self.indr2[iang - 1, :n]
        return blk, ang, r1, r2


# ---------------------------------------------------------------------------
# individual set-up steps
# ---------------------------------------------------------------------------

def input_grid(run):
    """Radial steps and Gauss-Legendre angles (mod_gridYpara_01y2.f:213-281)."""
    i = run.inp
    run.ah2 = (i.rfin2 - i.rmis2) / (i.npun2 - 1) if i.npun2 > 1 else 0.0
    run.ah1 = (i.rfin1 - i.rmis1) / (i.npun1 - 1) if i.npun1 > 1 else 0.0
    if i.inc not in (1, 2):
        raise ValueError("inc must be 1 or 2")
    if i.inc == 1 and i.j0 != 0:
        raise ValueError("inc=1 requires j0=0")
    run.nangu2 = i.nangu * i.inc
    if i.nangu == 1:
        run.cgamma = np.ones(1)
        run.wreal = np.ones(1)
        run._cgamprod = np.ones(1)
        run._weiprod = np.ones(1)
    else:
        w, x = gauleg(run.nangu2)
        run._cgamprod = x
        run._weiprod = w
        run.cgamma = x[: i.nangu].copy()
        run.wreal = w[: i.nangu] * i.inc
    if abs(i.iparity) != 1:
        raise ValueError("|iparity| must be 1")
    if i.jmax > (run.nangu2 - 1) * i.inc and i.npun2 > 1:
        raise ValueError("jmax > (nangu2-1)*inc")


def pot0(run):
    """Reduced masses and energy cut-offs (mod_pot_01y2.f:87-127)."""
    i = run.inp
    if i.radau != 0:
        raise NotImplementedError("Radau coordinates are not supported")
    xmtot = i.xm0 + i.xm1 + i.xm2
    run.xm1reac = i.xm0 * i.xm1 / (i.xm0 + i.xm1)
    run.xm2reac = i.xm2 * (i.xm0 + i.xm1) / xmtot if i.xm2 > 1e-3 else run.xm1reac
    run.xm1prod = i.xm0 * i.xm2 / (i.xm0 + i.xm2)
    run.xm2prod = i.xm1 * (i.xm0 + i.xm2) / xmtot
    run.xm1red = (i.xm0 * i.xm1) / (i.xm0 + i.xm1)
    run.xm2red = (i.xm2 * (i.xm0 + i.xm1)) / xmtot if i.xm2 > 1e-3 else run.xm1red
    run.vcutmax = i.vcutmaxev * C.eV2cm * C.conve1
    run.radcutmax = i.radcutmaxev * C.eV2cm * C.conve1
    run.rotcutmax = i.rotcutmaxev * C.eV2cm * C.conve1


def read_cont_pot(run, potdir):
    """Header of pot/cont.pot (written mod_pot_01y2.f:292-303, read :374-382)."""
    with open(os.path.join(potdir, "cont.pot")) as f:
        toks = f.read().split()
    p = 0
    nelec = int(toks[p]); p += 1
    run.nelec = nelec
    run.iomdiat = np.zeros(nelec, np.int32)
    run.iomatom = np.zeros(nelec, np.int32)
    run.sigdiat = np.zeros(nelec)
    run.sigatom = np.zeros(nelec)
    for e in range(nelec):
        run.iomdiat[e] = int(toks[p]); run.iomatom[e] = int(toks[p + 1])
        run.sigdiat[e] = float(toks[p + 2].replace("D", "E"))
        run.sigatom[e] = float(toks[p + 3].replace("D", "E")); p += 4
    vmin = float(toks[p].replace("D", "E")); maxpoint = int(toks[p + 1])
    vmaxtot = float(toks[p + 2].replace("D", "E")); p += 3
    xmis1, xfin1, mpun1 = float(toks[p]), float(toks[p + 1]), int(toks[p + 2]); p += 3
    xmis2, xfin2, mpun2 = float(toks[p]), float(toks[p + 1]), int(toks[p + 2]); p += 3
    mangu, minc = int(toks[p]), int(toks[p + 1]); p += 2
    i = run.inp
    npunreal = np.array([int(t) for t in toks[p:p + i.nangu]], np.int32)
    if (i.npun1 != mpun1 or i.npun2 != mpun2 or i.nangu != mangu or i.inc != minc):
        raise ValueError("input grid does not match the one used to generate pot/")
    if (abs(i.rmis1 - xmis1) > 1e-5 or abs(i.rfin1 - xfin1) > 1e-5
            or abs(i.rmis2 - xmis2) > 1e-5 or abs(i.rfin2 - xfin2) > 1e-5):
        raise ValueError("radial intervals do not match the ones used to generate pot/")
    if run.nelec != i.nelecmax:
        raise ValueError("nelec in cont.pot differs from nelecmax")
    run.vmintot = vmin
    run.vmaxtot = vmaxtot
    run.npunreal = npunreal
    run._maxpoint = maxpoint


def basis(run):
    """Omega/electronic channels and their j lists (mod_baseYfunciones_01y2.f:50-239)."""
    i = run.inp
    if i.xm2 < 1e-3:
        raise NotImplementedError("the diatom-only (Hdiatom) path is not supported")
    if i.iommax < i.iommin or i.iommax > i.Jtot:
        raise ValueError("bad iommin/iommax for Jtot")
    if i.inc == 2 and (-1) ** i.jref != (-1) ** i.j0:
        raise ValueError("j0 parity does not match jref")
    lmax = i.inc * (i.nangu - 1)
    iparbc = (-1) ** i.j0
    om, el, j00, noj, jb = [], [], [], [], []
    iommin_real = i.iommax
    for iom in range(i.iommin, i.iommax + 1):
        for ielec in range(1, run.nelec + 1):
            iomdi = int(run.iomdiat[ielec - 1])
            iomat = int(run.iomatom[ielec - 1])
            isign = -1 if i.Jtot % 2 != 0 else 1
            ipar = run.sigdiat[ielec - 1] * run.sigatom[ielec - 1] * isign
            if iom == 0 and iomdi == 0 and iomat == 0 and i.iparity != ipar:
                continue
            jmin = i.j0
            if i.inc == 2:
                jmin = 0 if run.sigdiat[ielec - 1] == iparbc else 1
            while jmin < abs(iom - iomat) or jmin < abs(iomdi):
                jmin += i.inc
            om.append(iom)
            el.append(ielec)
            j00.append(jmin)
            iommin_real = min(iommin_real, iom)
            js = [jmin + (k - 1) * i.inc for k in range(1, i.nangu + 1)]
            js = [j for j in js if j <= lmax]
            noj.append(len(js))
            jb.append(js + [0] * (i.nangu - len(js)))
    if iommin_real > i.iommin:
        raise ValueError("iommin must be set to %d" % iommin_real)
    if not om:
        raise ValueError("no channel in the basis")
    run.ncan = len(om)
    run.iombas = np.array(om, np.int32)
    run.nelebas = np.array(el, np.int32)
    run.j00 = np.array(j00, np.int32)
    run.nojbas = np.array(noj, np.int32)
    run.jbas = np.array(jb, np.int32)


def angular_functions(run):
    """Djmmp(iang,j,ielec,iom) = d^j_{Om-Om_at,Om_di}(gamma_i) sqrt((2j+1)/2 w_i)
    for iom = 0..Jtot (mod_baseYfunciones_01y2.f:454-551)."""
    i = run.inp
    lmax = (i.nangu - 1) * i.inc
    jmax2 = lmax * 2
    D = np.zeros((i.Jtot + 1, run.nelec, run.nangu2 + 1, i.nangu))
    for ielec in range(run.nelec):
        for iom in range(0, i.Jtot + 1):
            m2 = 2 * (iom - int(run.iomatom[ielec]))
            mp2 = 2 * int(run.iomdiat[ielec])
            mmax = max(m2, mp2) // 2
            jprin = max(mmax, i.jini)
            if i.nangu == 1:
                D[iom, ielec, jprin:lmax + 1, 0] = 1.0
                continue
            if iom > i.iommax + 1:
                continue          # only Omega <= iommax (+1 for the coupling bounds) is ever read
            gam = np.arccos(run._cgamprod[: i.nangu])
            pm = dwigner_vec(jmax2, m2, mp2, gam)
            for j in range(jprin, lmax + 1):
                xn = math.sqrt((2.0 * j + 1.0) * 0.5)
                D[iom, ielec, j, :] = pm[:, 2 * j] * xn * np.sqrt(run.wreal[: i.nangu])
    run.djmmp = D


def check_djmmp(run, criterj=1e-13):
    """Orthonormality self-check of the reference (mod_baseYfunciones_01y2.f:518-548);
    returns the largest deviation seen."""
    i = run.inp
    lmax = (i.nangu - 1) * i.inc
    worst = 0.0
    for b in range(run.ncan):
        e = run.nelebas[b] - 1
        om = run.iombas[b]
        js = [j for j in run.jbas[b, : run.nojbas[b]] if j <= lmax]
        M = run.djmmp[om, e][js] @ run.djmmp[om, e][js].T
        worst = max(worst, float(np.max(np.abs(M - np.eye(len(js))))))
    return worst


def radial_functions01_read(run, funcdir):
    """func/bcwf and func/eref (mod_baseYfunciones_01y2.f:837-923)."""
    i = run.inp
    nj = i.jmax - i.jini + 1
    nv = i.nvmax - i.nvini + 1
    run.nobc = np.zeros((run.nelec, nj), np.int32)
    run.ediat = np.zeros((run.nelec, nj, nv))
    run.fd = np.zeros((run.nelec, nj, nv, i.npun1))
    with open(os.path.join(funcdir, "bcwf")) as f:
        toks = f.read().split()
    p = 0
    for ielec in range(run.nelec):
        for j in range(i.jini, i.jmax + 1):
            p += 2
            nob = int(toks[p]); p += 1
            run.nobc[ielec, j - i.jini] = nob
            for iv in range(i.nvini, nob + 1):
                p += 1
                e = float(toks[p].replace("D", "E")); p += 1
                vals = np.array([float(t.replace("D", "E")) for t in toks[p:p + i.npun1]])
                p += i.npun1
                if iv <= i.nvmax:
                    run.ediat[ielec, j - i.jini, iv - i.nvini] = e
                    run.fd[ielec, j - i.jini, iv - i.nvini] = vals
    with open(os.path.join(funcdir, "eref")) as f:
        run.ediatref = float(f.read().split()[0].replace("D", "E"))
    for ielec in range(run.nelec):
        for j in range(i.jini, i.jmax + 1):
            nob = run.nobc[ielec, j - i.jini]
            for iv in range(i.nvini, min(nob, i.nvmax) + 1):
                run.ediat[ielec, j - i.jini, iv - i.nvini] -= run.ediatref


def product_radialf_read(path, jiniprod, jmaxprod, nviniprod, nvmaxprod, n2prod1, eref=None):
    """func/prodwf as the main program reads it (product_radialf_read,
    SRC/mod_baseYfunciones_01y2.f:1310-1400): per j its noBCprod (at most
    nvmaxprod) and n2prod1 (must be the input's), per v the energy,
    elecprodmax and vibelecprod and the n2prod1 x nelec function values.
    Energies are returned as stored, or less eref when it is given (the
    program subtracts func/eref).  Returns (fdprod[njp][nvp][nelec][n2prod1],
    ediatprod[njp][nvp], nobcprod[njp], elecprodmax[njp][nvp], vibelecprod[njp][nvp])."""
    njp, nvp = jmaxprod - jiniprod + 1, nvmaxprod - nviniprod + 1
    with open(path) as f:
        toks = f.read().split()
    p = 0
    fdprod = ediatprod = None
    nobcprod = np.zeros(njp, np.int32)
    elecprodmax = np.zeros((njp, nvp), np.int32)
    vibelecprod = np.zeros((njp, nvp), np.int32)
    for jj in range(njp):
        nob, nn2, nnelec = int(toks[p + 1]), int(toks[p + 2]), int(toks[p + 3])
        p += 4
        if nob > nvmaxprod:
            raise ValueError("noBCprod(%d) = %d exceeds nvmaxprod = %d" % (jiniprod + jj, nob, nvmaxprod))
        if nn2 != n2prod1:
            raise ValueError("n2prod1 = %d in func/prodwf but %d in the input" % (nn2, n2prod1))
        if fdprod is None:
            fdprod = np.zeros((njp, nvp, nnelec, n2prod1))
            ediatprod = np.zeros((njp, nvp))
        nobcprod[jj] = nob
        for iv in range(nviniprod, nob + 1):
            k = iv - nviniprod
            ediatprod[jj, k] = float(toks[p + 1].replace("D", "E"))
            elecprodmax[jj, k] = int(toks[p + 2])
            vibelecprod[jj, k] = int(float(toks[p + 3].replace("D", "E")))
            p += 4
            vals = [float(t.replace("D", "E")) for t in toks[p:p + n2prod1 * nnelec]]
            p += n2prod1 * nnelec
            fdprod[jj, k] = np.array(vals).reshape(n2prod1, nnelec).T
            if eref is not None:
                ediatprod[jj, k] -= eref
    return fdprod, ediatprod, nobcprod, elecprodmax, vibelecprod


def pot2(run, potdir):
    """Compressed grid, flat index and potential matrix; Chebyshev interval
    (mod_pot_01y2.f:344-533; interval :502-505)."""
    i = run.inp
    run.npuntot = int(run.npunreal.max())
    ne = run.nelec
    run.indr1 = np.zeros((i.nangu, run.npuntot), np.int32)
    run.indr2 = np.zeros((i.nangu, run.npuntot), np.int32)
    run.vvv = np.zeros((ne, ne, i.nangu, run.npuntot))
    for iang in range(1, i.nangu + 1):
        n = run.npunreal[iang - 1]
        path = os.path.join(potdir, "pot.%03d.dat" % iang)
        data = np.loadtxt(path, ndmin=2)
        if data.shape[0] < n or data.shape[1] != 2 + ne * ne:
            raise ValueError("truncated or malformed %s" % path)
        data = data[:n]
        run.indr1[iang - 1, :n] = data[:, 0].astype(np.int32)
        run.indr2[iang - 1, :n] = data[:, 1].astype(np.int32)
        col = 2
        for je in range(ne):          # Fortran order ((v(ie,je),ie),je)
            for ie in range(ne):
                run.vvv[je, ie, iang - 1, :n] = data[:, col]
                col += 1
        if (run.indr1[iang - 1, :n].min(initial=1) < 1 or run.indr1[iang - 1, :n].max(initial=1) > i.npun1
                or run.indr2[iang - 1, :n].min(initial=1) < 1 or run.indr2[iang - 1, :n].max(initial=1) > i.npun2):
            raise ValueError("grid index out of range in %s" % path)
    emaxtot = run.vmaxtot + run.radcutmax + 3.0 * run.rotcutmax
    run.delta2 = 0.5 * (emaxtot - run.vmintot)
    run.emindlt = run.vmintot + run.delta2
    # flat index (indtotproc for nproc=1)
    run.offs = np.zeros((i.nangu, run.ncan), np.int64)
    cnt = 0
    for iang in run.angle_order():
        for b in range(run.ncan):
            run.offs[iang - 1, b] = cnt
            cnt += int(run.npunreal[iang - 1])
    run.ntot = cnt


def rgauscolini(r, rcol, alpha, xk, factor):
    """sqrt(2) cos(k (r-r0)) N exp(-(r-r0)^2/alpha^2) (liboctdyn.f:2051-2066)."""
    g = math.cos((r - rcol) * xk) * math.sqrt(2.0)
    return g * factor * math.exp(-(r - rcol) * (r - rcol) / alpha / alpha)


def set_colini(run):
    """Initial collision packet in reactant Jacobi coordinates
    (mod_colini_01y2.f:25-177)."""
    i = run.inp
    if i.iprod == 1:
        raise NotImplementedError("product-Jacobi start (iprod=1) is not supported")
    run.rcolini = i.rcolini_ang
    ecol = i.ecol_ev * C.eV2cm * C.conve1
    deltae = i.deltae_ev * C.eV2cm * C.conve1
    run.xmasa0 = run.xm2reac
    run.xk0 = math.sqrt(2.0 * run.xmasa0 * ecol) / C.hbr
    run.alpha0 = math.sqrt(2.0 * ecol / run.xmasa0) * C.hbr / deltae
    run.factor0 = (2.0 / C.pi / run.alpha0 / run.alpha0) ** 0.25
    det = float(i.Jtot * (i.Jtot + 1) + i.jref * (i.jref + 1) - 2 * i.iomref * i.iomref)
    run.il0 = int(0.5 * (-1.0 + math.sqrt(1.0 + 4.0 * det)) + 0.5)
    s = 0.0
    for ir2 in range(1, i.npun2 + 1):
        r2 = i.rmis2 + (ir2 - 1) * run.ah2
        x = rgauscolini(r2, run.rcolini, run.alpha0, run.xk0, run.factor0)
        s += x * x
    run.gauss_norm = s * run.ah2
    psi = np.zeros(run.ntot)
    jref = i.jref
    for iang in run.angle_order():
        n = run.npunreal[iang - 1]
        for b in range(run.ncan):
            ielec = int(run.nelebas[b])
            iom = int(run.iombas[b])
            if ielec != i.ielecref:
                continue
            if i.iomref >= 0:
                angpart = run.djmmp[iom, ielec - 1, jref, iang - 1] if iom == i.iomref else 0.0
            else:
                angpart = ((-1.0) ** iom) * run.djmmp[iom, ielec - 1, jref, iang - 1] if iom <= jref else 0.0
            o = run.offs[iang - 1, b]
            ir1 = run.indr1[iang - 1, :n]
            ir2 = run.indr2[iang - 1, :n]
            rg = i.rmis2 + (ir2 - 1) * run.ah2
            fdi = np.ones(n) if i.npun1 == 1 else run.fd[i.ielecref - 1, jref - i.jini, i.nvref - i.nvini, ir1 - 1]
            g = np.cos((rg - run.rcolini) * run.xk0) * math.sqrt(2.0)
            xr2 = g * run.factor0 * np.exp(-(rg - run.rcolini) * (rg - run.rcolini) / run.alpha0 / run.alpha0)
            psi[o:o + n] = -xr2 * angpart * 1.0 * fdi * math.sqrt(run.ah2)
    run.psi0 = psi


def input_psie(run, inputfile):
    """&inputPsiE (SRC/mod_PsiE_01y2.f:19-88): with iphoto > 0, nofe energies
    (eV, one per line of file_resonancesE, relative to the input's directory)
    at which funE accumulates psi(E); sets run.efe_zot (zot), empty when off."""
    run.efe_zot = np.zeros(0)
    if run.inp.iphoto <= 0 or not inputfile:
        return
    g = namelist.read(inputfile).get("inputpsie", {})
    nofe = int(g.get("nofe", 0))
    if nofe <= 0:
        return
    path = os.path.join(os.path.dirname(os.path.abspath(inputfile)), str(g.get("file_resonancese", "")))
    with open(path) as f:
        vals = [float(t.replace("D", "E").replace("d", "e")) for t in f.read().split()[:nofe]]
    if len(vals) < nofe:
        raise ValueError("%s holds fewer than nofe = %d energies" % (path, nofe))
    run.efe_zot = np.array(vals) * C.eV2cm * C.conve1


def load_sweep(inputfile, Js, overrides):
    """Partial waves that share one grid, potential and diatomic functions:
    the files are read once; ``overrides(J)`` gives the per-J namelist values
    (Jtot, iparity, iommin, iommax, iomref)."""
    import copy
    base = load(inputfile)
    runs = []
    for J in Js:
        inp = copy.copy(base.inp)
        for k, v in overrides(J).items():
            setattr(inp, k, v)
        r = copy.copy(base)
        r.inp = inp
        basis(r)
        angular_functions(r)
        # flat layout depends on the number of blocks
        r.offs = np.zeros((inp.nangu, r.ncan), np.int64)
        cnt = 0
        for iang in r.angle_order():
            for b in range(r.ncan):
                r.offs[iang - 1, b] = cnt
                cnt += int(r.npunreal[iang - 1])
        r.ntot = cnt
        if inp.iphoto == 0:
            set_colini(r)
        runs.append(r)
    return runs


def load(inputfile, potdir=None, funcdir=None, inputs=None):
    """Run the host set-up in the order main_madwave3.f does (:130-185)."""
    base = os.path.dirname(os.path.abspath(inputfile)) if inputfile else "."
    inp = inputs if inputs is not None else Inputs.read(inputfile)
    potdir = potdir or os.path.join(base, "pot")
    funcdir = funcdir or os.path.join(base, "func")
    run = Run(inp=inp)
    input_grid(run)
    pot0(run)
    read_cont_pot(run, potdir)
    basis(run)
    angular_functions(run)
    radial_functions01_read(run, funcdir)
    pot2(run, potdir)
    if inp.iphoto == 0:
        set_colini(run)
    input_psie(run, inputfile)
    return run
