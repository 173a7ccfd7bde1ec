"""Set-up of the product-state projection for iprod = 2 (ini_transcoor,
SRC/mod_coortrans01_02.f:32-690): the tables the device projection takes
(``madwave3_gb300.product.ProductProjection``) from the grid, the masses and
the product diatom's radial functions.

* ``trans_rg_jac``: changeini's first part (:283-360) -- for every stored point
  of the projection's angles, the sine-basis interpolation from the point's r1
  to the r1 at which the product Jacobi distance equals Rbalinprod, with the
  Jacobian of the change of variables.
* ``prod_functions``: prodwftrans (:485-588) -- each product state
  (v', j', Omega') as a function of the reactant (R, gamma): the product
  radial function splined at the product diatom distance, times the Wigner
  function of the angle between the product Jacobi vectors and the Jacobian.
* ``dtrans``: bfreac2prod (:592-690) -- the body-fixed rotation from reactant to
  product Omega, d^J_{Omega,Omega'} of the angle between the two R vectors
  with the parity combination.
* ``s2prodfac``: ini_transcoor's collision factor (:121-145).

The product radial functions, their energies and noBCprod come from the
reference's product_radialf_read (SRC/mod_baseYfunciones_01y2.f:1085-1250),
which reads them from the func/ files; here they are arguments.

The spline is the reference's (SPLSET / SPLINQQ / DLAGRA / JORDAN,
SRC/liboctdyn.f:298-400, 926-990): a cubic Hermite spline whose end
derivatives come from four-point Lagrange polynomials and whose inner
derivatives solve the usual tridiagonal system, with the reference's
R^-6 / R^-8 extension beyond the last point.
"""
import math

import numpy as np

from .wigner import dwigner, dwigner_vec


# ---------------------------------------------------------------------------
# the reference's spline (SRC/liboctdyn.f)
# ---------------------------------------------------------------------------
def dlagra(x, y, ip):
    """DLAGRA (liboctdyn.f:960-985): derivative at x[ip] of the Lagrange
    polynomial through (x, y) (ip 0-based)."""
    n = len(x)
    d = 0.0
    for i in range(n):
        if i == ip:
            continue
        yp = y[i]
        for j in range(n):
            if j != ip and j != i:
                yp = yp * (x[ip] - x[j])
        for j in range(n):
            if j != i:
                yp = yp / (x[i] - x[j])
        d = d + yp
    for i in range(n):
        if i != ip:
            d = d + y[ip] / (x[ip] - x[i])
    return d


def jordan(mu, lam, b):
    """JORDAN (liboctdyn.f:926-958): solves lam_i x_{i-1} + 2 x_i + mu_i x_{i+1} = b_i."""
    n = len(b)
    b = np.array(b, np.float64)
    piv = np.empty(n)
    piv[0] = 2.0
    for i in range(1, n):
        piv[i] = 2.0 - lam[i] * mu[i - 1] / piv[i - 1]
        b[i] = b[i] - lam[i] / piv[i - 1] * b[i - 1]
    x = np.empty(n)
    x[n - 1] = b[n - 1] / piv[n - 1]
    for i in range(n - 2, -1, -1):
        x[i] = (b[i] - x[i + 1] * mu[i]) / piv[i]
    return x


def splset(f, x):
    """SPLSET (liboctdyn.f:342-400): the derivatives at the knots."""
    f = np.asarray(f, np.float64)
    x = np.asarray(x, np.float64)
    nx = len(x)
    hx = x[1:] - x[:-1]
    rl = hx[1:] / (hx[:-1] + hx[1:])                 # lambda_i, i = 1..nx-2
    rm = 1.0 - rl
    p0 = dlagra(x[:4], f[:4], 0)
    pn = dlagra(x[nx - 4:], f[nx - 4:], 3)
    b = 3.0 * rl / hx[:-1] * (f[1:-1] - f[:-2]) + 3.0 * rm / hx[1:] * (f[2:] - f[1:-1])
    b[0] = b[0] - rl[0] * p0
    b[-1] = b[-1] - rm[-1] * pn
    d = np.empty(nx)
    d[0], d[-1] = p0, pn
    d[1:-1] = jordan(rm, rl, b)
    return d


def splinqq(f, d, x, r, iold=1):
    """SPLINQQ (liboctdyn.f:298-340) at r, searching from knot iold (0-based
    index of the reference's IOLD = 2 is 1)."""
    nx = len(x)
    if r >= x[nx - 1]:
        ro, yo, yp = x[nx - 1], f[nx - 1], d[nx - 1]
        ain = yo + yp * ro / 6.0
        c8 = -ain * 3.0 * ro ** 8
        c6 = yo * ro ** 6 - c8 / ro / ro
        return c6 / r ** 6 + c8 / r ** 8
    idol = iold
    while idol < nx and not (r < x[idol]):
        idol += 1
    hi = x[idol] - x[idol - 1]
    xr = (r - x[idol - 1]) / hi
    u1 = xr * xr * (-2.0 * xr + 3.0)
    u3 = hi * xr * xr * (xr - 1.0)
    u2 = 1.0 - u1
    u4 = hi * xr * ((xr - 2.0) * xr + 1.0)
    return u1 * f[idol] + u2 * f[idol - 1] + u3 * d[idol] + u4 * d[idol - 1]


def splinqq_vec(f, d, x, rr):
    """splinqq at many points at once (each searched from the second knot, as
    the reference does for increasing points)."""
    f = np.asarray(f, np.float64)
    d = np.asarray(d, np.float64)
    x = np.asarray(x, np.float64)
    rr = np.asarray(rr, np.float64)
    nx = len(x)
    out = np.empty(rr.shape)
    tail = rr >= x[nx - 1]
    if tail.any():
        ro, yo, yp = x[nx - 1], f[nx - 1], d[nx - 1]
        ain = yo + yp * ro / 6.0
        c8 = -ain * 3.0 * ro ** 8
        c6 = yo * ro ** 6 - c8 / ro / ro
        rt = rr[tail]
        out[tail] = c6 / rt ** 6 + c8 / rt ** 8
    r = rr[~tail]
    idol = np.maximum(1, np.searchsorted(x, r, side="right"))
    hi = x[idol] - x[idol - 1]
    xr = (r - x[idol - 1]) / hi
    u1 = xr * xr * (-2.0 * xr + 3.0)
    u3 = hi * xr * xr * (xr - 1.0)
    u2 = 1.0 - u1
    u4 = hi * xr * ((xr - 2.0) * xr + 1.0)
    out[~tail] = u1 * f[idol] + u2 * f[idol - 1] + u3 * d[idol] + u4 * d[idol - 1]
    return out


# ---------------------------------------------------------------------------
# mass factors of the reactant -> product Jacobi change
# ---------------------------------------------------------------------------
def _ab(inp):
    xm0, xm1, xm2 = inp.xm0, inp.xm1, inp.xm2
    a = (xm0 + xm2) / xm2 - xm1 / (xm0 + xm1)
    b = (xm0 + xm1) / xm1 - xm2 / (xm0 + xm2)
    return a, b


def _geometry(inp, rga, cg, rgb):
    """(rpa, rpb) for reactant R = rga, cos(gamma) = cg and product R = rgb, or
    None where the square root is imaginary (prodwftrans :530-541)."""
    a, _ = _ab(inp)
    xm0, xm1, xm2 = inp.xm0, inp.xm1, inp.xm2
    sqr = rga * rga * (cg * cg - 1.0) + (rgb * (xm0 + xm2) / xm2) ** 2
    if not sqr > 0.0:
        return None
    rpa = (rga * cg + math.sqrt(sqr)) / a
    rpb = (rpa * xm1 / (xm0 + xm1)) ** 2 + rga * rga + 2.0 * rpa * rga * cg * xm1 / (xm0 + xm1)
    return rpa, math.sqrt(rpb)


def trans_rg_jac(run, rbalinprod, nangproj0, nangproj1):
    """changeini :283-360: transRgjac on the wave's state vector layout (0 on
    the points of angles outside [nangproj0, nangproj1])."""
    inp = run.inp
    n1, n2 = inp.npun1, inp.npun2
    ah1, ah2 = run.ah1, run.ah2
    a, _ = _ab(inp)
    xm0, xm2 = inp.xm0, inp.xm2
    # sinmom (liboctdyn.f:1004-1031): p_m = 2 pi m / (2 (npun1 + 1) ah1)
    xk = 2.0 * math.pi * np.arange(1, n1 + 1) / (2.0 * (n1 + 1.0) * ah1)
    r1 = inp.rmis1 + np.arange(n1) * ah1
    out = np.zeros(run.ntot)
    c0 = (xm0 + xm2) * rbalinprod / xm2
    s1 = np.sin(np.outer(r1, xk))
    for iang in range(nangproj0, nangproj1 + 1):
        cg = run.cgamma[iang - 1]
        raux = np.zeros((n2, n1))
        for ir2 in range(n2):
            r2 = inp.rmis2 + ir2 * ah2
            x2 = r2 * r2 * (cg * cg - 1.0)
            if not c0 * c0 + x2 > 0.0:
                continue
            r1inter = (r2 * cg + math.sqrt(c0 * c0 + x2)) / a
            if not (inp.rmis1 < r1inter < inp.rfin1):
                continue
            s = s1 @ np.sin(xk * r1inter)
            jac1 = math.sqrt(x2 + (rbalinprod * (xm0 + xm2) / xm2) ** 2)
            jac = math.sqrt(rbalinprod * ((xm0 + xm2) / xm2) ** 2 / (a * jac1))
            raux[ir2] = s * 2.0 / (n1 + 1.0) * jac / math.sqrt(ah1)
        n = run.npunreal[iang - 1]
        i1 = run.indr1[iang - 1, :n] - 1
        i2 = run.indr2[iang - 1, :n] - 1
        for b in range(run.ncan):
            o = run.offs[iang - 1, b]
            out[o:o + n] = raux[i2, i1]
    return out


def prod_functions(run, rbalinprod, fdprod, n2prod0, n2prod1, nangproj0, nangproj1, iom, j, iv):
    """prodwftrans (:485-588) for one product state: prodaux[nelec][nang][n2p].
    fdprod[nelec][n2prod1]: the state's radial function on the R grid's first
    n2prod1 points (fdprod(ir2, iv, j, ielec))."""
    inp = run.inp
    _, bm = _ab(inp)
    xm0, xm1 = inp.xm0, inp.xm1
    lmax = (inp.nangu - 1) * inp.inc
    jmax2 = lmax * 2
    facnorm = 1.0 / math.sqrt(2.0) if inp.inc == 2 else 1.0
    xx = inp.rmis2 + np.arange(n2prod1) * run.ah2
    nang, n2p = nangproj1 - nangproj0 + 1, n2prod1 - n2prod0 + 1
    out = np.zeros((run.nelec, nang, n2p))
    rgb = rbalinprod
    for ielec in range(run.nelec):
        ff = np.asarray(fdprod[ielec][:n2prod1], np.float64)
        dd = splset(ff, xx)
        for ia, iang in enumerate(range(nangproj0, nangproj1 + 1)):
            cg = run.cgamma[iang - 1]
            w = run._weiprod[iang - 1]
            for k, irga in enumerate(range(n2prod0, n2prod1 + 1)):
                rga = inp.rmis2 + (irga - 1) * run.ah2
                g = _geometry(inp, rga, cg, rgb)
                if g is None:
                    continue
                rpa, rpb = g
                fdiat = 0.0
                if inp.rmis2 <= rpb <= inp.rfin2:
                    fdiat = splinqq(ff, dd, xx, rpb)
                angjac = (rgb * rgb + bm * bm * rpb * rpb - (rga * (xm0 + xm1) / xm1) ** 2) * 0.5 / (bm * rpb * rgb)
                if abs(angjac) > 1.0:
                    continue
                beta = math.acos(angjac)
                pm = dwigner(jmax2, 2 * (iom - int(run.iomatom[ielec])), 2 * int(run.iomdiat[ielec]), beta)
                xn = math.sqrt((2.0 * j + 1.0) * 0.5)
                angpart = pm[2 * j] * xn * math.sqrt(w) * facnorm
                xjac1 = rga ** 2 * (cg ** 2 - 1.0) + (rgb * (xm0 + inp.xm2) / inp.xm2) ** 2
                a, _ = _ab(inp)
                xjaco = rgb * ((xm0 + inp.xm2) / inp.xm2) ** 2 / (a * math.sqrt(xjac1))
                out[ielec, ia, k] = fdiat * angpart * rga * rpa * math.sqrt(xjaco) / (rpb * rgb)
    return out


def prod_geometry(run, rbalinprod, n2prod0, n2prod1, nangproj0, nangproj1):
    """The per-(angle, R) quantities of prodwftrans (:485-588) that do not depend
    on the product state: [nang][n2p] arrays of rpa, rpb, beta, the factor
    rga rpa sqrt(xjaco) / (rpb rgb) and a mask of the points that contribute
    (real square root, |cos beta| <= 1)."""
    inp = run.inp
    a, bm = _ab(inp)
    xm0, xm1, xm2 = inp.xm0, inp.xm1, inp.xm2
    rgb = rbalinprod
    cg = np.asarray(run.cgamma[nangproj0 - 1:nangproj1], np.float64)[:, None]
    rga = (inp.rmis2 + np.arange(n2prod0 - 1, n2prod1) * run.ah2)[None, :]
    with np.errstate(invalid="ignore", divide="ignore"):
        sqr = rga * rga * (cg * cg - 1.0) + (rgb * (xm0 + xm2) / xm2) ** 2
        ok = sqr > 0.0
        rpa = (rga * cg + np.sqrt(np.where(ok, sqr, 1.0))) / a
        rpb = np.sqrt((rpa * xm1 / (xm0 + xm1)) ** 2 + rga * rga + 2.0 * rpa * rga * cg * xm1 / (xm0 + xm1))
        angjac = (rgb * rgb + bm * bm * rpb * rpb - (rga * (xm0 + xm1) / xm1) ** 2) * 0.5 / (bm * rpb * rgb)
        ok &= np.abs(angjac) <= 1.0
        beta = np.arccos(np.clip(angjac, -1.0, 1.0))
        xjac1 = rga ** 2 * (cg ** 2 - 1.0) + (rgb * (xm0 + xm2) / xm2) ** 2
        xjaco = rgb * ((xm0 + xm2) / xm2) ** 2 / (a * np.sqrt(np.where(ok, xjac1, 1.0)))
        fac = rga * rpa * np.sqrt(np.where(ok, xjaco, 0.0)) / (rpb * rgb)
    return rpa, rpb, beta, np.where(ok, fac, 0.0), ok


def prod_functions_omega(run, rbalinprod, fdprod, nobcprod, jiniprod, jmaxprod, nviniprod, n2prod0, n2prod1,
                         nangproj0, nangproj1, iom):
    """prodwftrans for every product state (j, v) of one Omega at once:
    [njp][nvp][nelec][nang][n2p] (zero for j < Omega and v > noBCprod(j)).
    Same arithmetic as prod_functions, vectorised over the (angle, R) points."""
    inp = run.inp
    lmax = (inp.nangu - 1) * inp.inc
    jmax2 = lmax * 2
    facnorm = 1.0 / math.sqrt(2.0) if inp.inc == 2 else 1.0
    xx = inp.rmis2 + np.arange(n2prod1) * run.ah2
    rpa, rpb, beta, fac, ok = prod_geometry(run, rbalinprod, n2prod0, n2prod1, nangproj0, nangproj1)
    nang, n2p = ok.shape
    w = np.asarray(run._weiprod[nangproj0 - 1:nangproj1], np.float64)[:, None]
    inside = ok & (rpb >= inp.rmis2) & (rpb <= inp.rfin2)
    njp = jmaxprod - jiniprod + 1
    nvp = int(np.max(np.asarray(fdprod).shape[1])) if njp else 0
    out = np.zeros((njp, nvp, run.nelec, nang, n2p))
    for ielec in range(run.nelec):
        pm = dwigner_vec(jmax2, 2 * (iom - int(run.iomatom[ielec])), 2 * int(run.iomdiat[ielec]),
                         beta[ok]).T                                   # [jmax2+1][npts]
        for j in range(max(jiniprod, iom), jmaxprod + 1):
            jj = j - jiniprod
            ang = np.zeros((nang, n2p))
            ang[ok] = pm[2 * j] * math.sqrt((2.0 * j + 1.0) * 0.5)
            ang = ang * np.sqrt(w) * facnorm
            for iv in range(nviniprod, int(nobcprod[jj]) + 1):
                ff = np.asarray(fdprod[jj][iv - nviniprod][ielec][:n2prod1], np.float64)
                dd = splset(ff, xx)
                fdiat = np.zeros((nang, n2p))
                fdiat[inside] = splinqq_vec(ff, dd, xx, rpb[inside])
                out[jj, iv - nviniprod, ielec] = np.where(ok, fdiat * ang * fac, 0.0)
    return out


def dtrans(run, rbalinprod, n2prod0, n2prod1, nangproj0, nangproj1, iomminprod, iommaxprod):
    """bfreac2prod (:592-690): dtrans[ncan][nom][nang][n2p]."""
    inp = run.inp
    if iommaxprod > inp.Jtot:
        raise ValueError("iommaxprod > Jtot")
    a, bm = _ab(inp)
    xm0, xm1 = inp.xm0, inp.xm1
    nang, n2p, nom = nangproj1 - nangproj0 + 1, n2prod1 - n2prod0 + 1, iommaxprod - iomminprod + 1
    out = np.zeros((run.ncan, nom, nang, n2p))
    rgb = rbalinprod
    if inp.Jtot == 0:
        out[:] = 1.0
        return out
    jt2 = 2 * inp.Jtot
    for ia, iang in enumerate(range(nangproj0, nangproj1 + 1)):
        cg = run.cgamma[iang - 1]
        for k, ir in enumerate(range(n2prod0, n2prod1 + 1)):
            rga = inp.rmis2 + (ir - 1) * run.ah2
            g = _geometry(inp, rga, cg, rgb)
            if g is None:
                continue
            _, rpb = g
            angjac = (rgb * rgb + bm * bm * rpb * rpb - (rga * (xm0 + xm1) / xm1) ** 2) * 0.5 / (bm * rpb * rgb)
            if abs(angjac) > 1.0:
                continue
            angb = math.acos(angjac)
            deno = (bm * rpb) ** 2 + rgb * rgb - 2.0 * bm * rpb * rgb * math.cos(angb)
            ctrans = (bm * rpb * math.cos(angb) - rgb) / math.sqrt(deno)
            if abs(ctrans) > 1.0:
                continue
            at = math.acos(ctrans)
            for b in range(run.ncan):
                omr = int(run.iombas[b])
                for o, omp in enumerate(range(iomminprod, iommaxprod + 1)):
                    x1 = dwigner(jt2, 2 * omr, 2 * omp, at)[jt2]
                    if omr != 0:
                        ss = float(inp.iparity) * (-1.0) ** abs(inp.Jtot + omr)
                        x1 = (x1 + ss * dwigner(jt2, -2 * omr, 2 * omp, at)[jt2]) / math.sqrt(2.0)
                    if omp != 0:
                        x1 = x1 * math.sqrt(2.0)
                    out[b, o, ia, k] = x1
    return out


def s2prodfac(run, etot, apaqini, ediatprod, nobcprod, nviniprod, nvmaxprod):
    """ini_transcoor :121-145 (iphoto = 0): S2prodfac[njp][nvp][netot] =
    hbar^2 p_fin p_ini / (2 apaqini) / (mu_reac mu_prod), 0 where apaqini < 1e-10.
    ediatprod[njp][nvp] in zot, nobcprod[njp] = noBCprod(jiniprod:jmaxprod)."""
    from .constants import hbr

    etot = np.asarray(etot, np.float64)
    apaqini = np.asarray(apaqini, np.float64)
    njp = len(nobcprod)
    out = np.zeros((njp, nvmaxprod - nviniprod + 1, etot.size))
    pini = np.sqrt(np.where(etot > 0.0, etot, 0.0) * run.xmasa0 * 2.0 / hbr / hbr)
    ok = apaqini >= 1e-10
    for jj in range(njp):
        for iv in range(nviniprod, int(nobcprod[jj]) + 1):
            ek = etot - ediatprod[jj][iv - nviniprod]
            pfin = np.sqrt(np.where(ek > 0.0, ek, 0.0) * run.xm2prod * 2.0 / hbr / hbr)
            f = hbr * hbr * pfin * pini / (2.0 * np.where(ok, apaqini, 1.0)) / run.xmasa0 / run.xm2prod
            out[jj, iv - nviniprod] = np.where(ok, f, 0.0)
    return out


def ini_transcoor(run, rbalinprod, n2prod0, n2prod1, nangproj0, nangproj1, iomminprod, iommaxprod, jiniprod,
                  jmaxprod, nviniprod, nvmaxprod, nobcprod, fdprod):
    """changeini (:211-483): the ProductProjection for the device.
    fdprod[njp][nvp][nelec][n2prod1] (fdprod(ir2, iv, j, ielec) of the
    reference), nobcprod[njp] = noBCprod(jiniprod:jmaxprod)."""
    from ..product import ProductProjection

    njp, nvp = jmaxprod - jiniprod + 1, nvmaxprod - nviniprod + 1
    nom = iommaxprod - iomminprod + 1
    nang, n2p = nangproj1 - nangproj0 + 1, n2prod1 - n2prod0 + 1
    wf = np.zeros((nom, njp, nvp, run.nelec, nang, n2p))
    for o, iom in enumerate(range(iomminprod, iommaxprod + 1)):
        wf[o] = prod_functions_omega(run, rbalinprod, fdprod, nobcprod, jiniprod, jmaxprod, nviniprod, n2prod0,
                                     n2prod1, nangproj0, nangproj1, iom)
    return ProductProjection(
        n2prod0, n2prod1, nangproj0, nangproj1, iomminprod, iommaxprod, jiniprod, jmaxprod, nviniprod, nvmaxprod,
        np.asarray(nobcprod, np.int32), trans_rg_jac(run, rbalinprod, nangproj0, nangproj1),
        dtrans(run, rbalinprod, n2prod0, n2prod1, nangproj0, nangproj1, iomminprod, iommaxprod), wf)
