"""pot.out: the pre-processing program that tabulates a surface for madwave3.

Restates the parts of ``pot.out`` (SRC/main_potini.f:25-104) that the
propagation reads, for a surface given as a ``potelebond(r1, r2, cos)``
callable returning the diabatic matrix in hartree (the interface of the
reference's pothead.f files):

* ``radial_functions01_write`` (SRC/mod_baseYfunciones_01y2.f:553-836): the
  reactant diatom's rovibrational levels on a 2000-point grid -- finite
  difference eigenvalues as starting energies, Numerov-Cooley refinement
  (``schr``, SRC/liboctdyn.f:405-587), spline interpolation onto the
  propagation's r1 grid (SPLSET/SPLINQQ) and normalisation -- written to
  ``func/bcwf`` and ``func/eref``;
* ``pot1`` (SRC/mod_pot_01y2.f:147-341): the surface on the reactant Jacobi
  grid, referred to ``eref``, kept where an adiabatic energy lies below Vcut,
  written to ``pot/pot.NNN.dat`` and ``pot/cont.pot``.

The finite-difference eigenvalues come from LAPACK's tridiagonal solver where
the reference calls Numerical Recipes' TQLI (SRC/liboctdyn.f:233-296); they
only seed the Numerov iterations, which converge to the same levels.
"""
import math
import os

import numpy as np
from scipy.linalg import eigvalsh_tridiagonal

from . import constants as C
from . import namelist
from .setup import Inputs, input_grid, pot0
from .transcoor import splset

NPUNT = 2000        # radial_functions01_write's grid


def _sqrt(x):
    return math.sqrt(x) if x >= 0.0 else float("nan")


def schr(e0, rmin, rmax, n, maxit, eps, v):
    """SCHR (SRC/liboctdyn.f:405-587): Numerov-Cooley eigenvalue refinement of
    -p'' + v p = e p on n points of [rmin, rmax] (v and e in the units of
    2 m E).  Inward integration from rmax to the matching point (the first
    maximum of |p| coming in), outward from rmin, Cooley's energy correction,
    repeated until the correction stops shrinking and is below eps.
    Returns (e2, nodes, p) with p normalised to sum p^2 h = 1."""
    h = (rmax - rmin) / float(n - 1)
    h2 = h ** 2
    hv = h2 / 12.0
    e = e0
    test = -1.0
    de = 0.0
    dold = 0.0
    p = [0.0] * (n + 1)           # 1-based as the Fortran arrays
    V = [0.0] + list(v)
    df = 0.0
    for _ in range(maxit):
        # inward integration, first steps
        p[n] = 1.0e-30
        gn = V[n] - e
        gi = V[n - 1] - e
        if not gi >= 0.0:
            e = V[n - 2]
        apr = (rmax - h) * _sqrt(gi) - rmax * _sqrt(gn)
        if apr > 50.0:
            apr = 50.0
        p[n - 1] = p[n] * math.exp(-apr) if apr == apr else float("nan")
        y1 = (1.0 - hv * gn) * p[n]
        y2 = (1.0 - hv * gi) * p[n - 1]
        m = n - 2
        while True:
            y3 = y2 + ((y2 - y1) + h2 * gi * p[m + 1])
            gi = V[m] - e
            p[m] = y3 / (1.0 - hv * gi)
            if not abs(p[m]) < 1.0e34:
                if p[m] != p[m]:
                    pass              # NaN: the reference carries it on
                else:
                    pm = p[m + 1]
                    for j in range(m + 1, n + 1):
                        p[j] = p[j] / pm
                    y1, y2, y3 = y1 / pm, y2 / pm, y3 / pm
                    gi = V[m + 1] - e
                    continue
            if abs(p[m]) <= abs(p[m + 1]) or m <= 2:
                break
            y1, y2 = y2, y3
            m -= 1
        pm = p[m]
        yin = y2 / pm
        for j in range(m, n + 1):
            p[j] = p[j] / pm
        # outward integration
        p[1] = 1.0
        y1 = 0.0
        gi = V[1] - e
        y2 = (1.0 - hv * gi) * p[1]
        i = 2
        while i <= m:
            y3 = y2 + ((y2 - y1) + h2 * gi * p[i - 1])
            gi = V[i] - e
            p[i] = y3 / (1.0 - hv * gi)
            if not abs(p[i]) < 1.0e34 and p[i] == p[i]:
                i1 = i - 1
                pm = p[i1]
                for j in range(1, i1 + 1):
                    p[j] = p[j] / pm
                y1, y2, y3 = y1 / pm, y2 / pm, y3 / pm
                gi = V[i1] - e
                continue          # label 110: the same point again
            y1, y2 = y2, y3
            i += 1
        pm = p[m]
        if pm == 0.0:
            # label 149 is reached before DOLD = DE: the old DOLD is kept
            f = 9.99999e29
            df = -f
            de = abs(0.0001 * e)
        else:
            yout = y1 / pm
            ym = y3 / pm
            for j in range(1, m + 1):
                p[j] = p[j] / pm
            df = 0.0
            for j in range(1, n + 1):
                df = df - p[j] ** 2
            f = (-yout - yin + 2.0 * ym) / h2 + (V[m] - e)
            dold = de
            if abs(f) < 1.0e37:
                de = -f / df
            else:
                f = 9.99999e29
                df = -f
                de = abs(0.0001 * e)
        eold = e
        e = e + de
        test = max(abs(dold) - abs(de), test)
        if test < 0.0:
            continue
        if abs(e - eold) < eps:
            break
    # node count (labels 173-192)
    kv = 0
    for j in range(3, n - 1):
        pj, pjm, pjp, pjm2 = p[j], p[j - 1], p[j + 1], p[j - 2]
        if pj >= 0.0:
            if pjm < 0.0 and pjp >= 0.0 and pjm2 < 0.0:
                kv += 1
        else:
            if pjm > 0.0:
                if pjp < 0.0 and pjm2 >= 0.0:
                    kv += 1
            elif pjm == 0.0:
                if pjp < 0.0 and pjm2 > 0.0:
                    kv += 1
    sn = _sqrt(-h * df)
    return e, kv, [x / sn for x in p[1:]]


def splinqq_many(f, d, x, rr):
    """SPLINQQ (SRC/liboctdyn.f:298-340) at increasing points rr: the cubic
    Hermite piece of the first knot above r (searched from the second knot),
    or the C6/r^6 + C8/r^8 tail at and beyond the last knot."""
    rr = np.asarray(rr, np.float64)
    nx = len(x)
    out = np.empty(rr.size)
    for k, r in enumerate(rr):
        if r >= x[nx - 1]:
            ro, yo, yp = x[nx - 1], f[nx - 1], d[nx - 1]
            ain = yo + yp * ro / 6.0
            c8 = -ain * 3.0 * ro ** 8
            c6 = yo * ro ** 6 - c8 / ro / ro
            out[k] = c6 / r ** 6 + c8 / r ** 8
            continue
        idol = max(1, int(np.searchsorted(x, r, side="right")))
        hi = x[idol] - x[idol - 1]
        xr = (r - x[idol - 1]) / hi
        u1 = xr * xr * (-2.0 * xr + 3.0)
        u3 = hi * xr * xr * (xr - 1.0)
        u2 = 1.0 - u1
        u4 = hi * xr * ((xr - 2.0) * xr + 1.0)
        out[k] = u1 * f[idol] + u2 * f[idol - 1] + u3 * d[idol] + u4 * d[idol - 1]
    return out


def _inputs(path_or_groups):
    groups = namelist.read(path_or_groups) if isinstance(path_or_groups, str) else path_or_groups
    inp = Inputs.from_namelists(groups)
    flat = {}
    for g in groups.values():
        flat.update(g)
    return inp, flat


class _Grid:
    pass


def _grid(inp):
    g = _Grid()
    g.inp = inp
    input_grid(g)
    pot0(g)
    return g


def radial_functions01_write(g, potelebond, r2inf=100.0, nelec=1, bound_test="margin"):
    """Reactant (01) diatom levels and functions on the propagation's r1 grid
    (SRC/mod_baseYfunciones_01y2.f:553-836).  Returns (nobc[nelec][nj],
    ediat[nelec][nj][nv] in zot, fd[nelec][nj][nv][npun1], ediatref).

    ``bound_test`` picks which levels count as bound.  "margin" is the shipped
    source: E more than 0.01 hartree below V at the grid's end (:702), level
    counts starting at nvini - 1 (:584) and the j loop ending at the first j
    with at most one level whose last v failed (:758).  "below_asymptote" is
    the earlier form the same routine has in SRC/mod_baseYfunciones_Renner_01y2.f
    (:567, :684, :737) and in the comment at :701: E below V at the grid's
    end, counts starting at 0 and the loop ending at a j whose count stayed 0;
    the shipped H + HD run (EXAMPLES/HD+H_collision/J000-check) was made with
    it (its log lists the j = 37..39 entries that only a count of 0 leaves)."""
    if bound_test not in ("margin", "below_asymptote"):
        raise ValueError("bound_test must be 'margin' or 'below_asymptote'")
    inp = g.inp
    n1 = inp.npun1
    nj = inp.jmax - inp.jini + 1
    nv = inp.nvmax - inp.nvini + 1
    nobc = np.full((nelec, nj), inp.nvini - 1 if bound_test == "margin" else 0, np.int32)
    ediat = np.zeros((nelec, nj, nv))
    fd = np.zeros((nelec, nj, nv, n1))
    rmis = inp.rmis1 / C.convl
    rfin = (inp.rmis1 + float(n1 - 1) * g.ah1) / C.convl
    ah = (rfin - rmis) / float(NPUNT - 1)
    rg = r2inf / C.convl
    xm = g.xm1reac * C.convm
    xz = 0.5 / xm
    r = rmis + np.arange(NPUNT, dtype=np.float64) * ah
    r1grid = np.array([(inp.rmis1 + float(ir1) * g.ah1) / C.convl for ir1 in range(n1)])
    for ie in range(nelec):
        V = potelebond(r, np.full(NPUNT, rg), 1.0)[ie, ie]
        irmin = 0
        vmin = 1e10
        for ir in range(NPUNT):
            if V[ir] < vmin:
                vmin = V[ir]
                irmin = ir
        if irmin == 0:
            continue                       # repulsive state: no bound levels
        for jj, j in enumerate(range(inp.jini, inp.jmax + 1)):
            xl = 0.5 * float(j * (j + 1)) / xm
            vv = V + xl / r / r
            diag = -2.0 - 2.0 * xm * vv * ah * ah
            lam = eigvalsh_tridiagonal(diag, np.ones(NPUNT - 1))
            alpha = np.sort(-xz * lam / ah / ah)
            ifail = -1
            for iv in range(inp.nvini, inp.nvmax + 1):
                ifail = -1
                if (V[NPUNT - 1] - alpha[iv] > 1.0e-2) if bound_test == "margin" else (alpha[iv] < V[NPUNT - 1]):
                    xz1 = 2.0 * xm
                    e0 = alpha[iv] * xz1
                    vvs = (vv * xz1).tolist()
                    e2, _, p = schr(e0, rmis, rfin, NPUNT, 20, 1.0e-10, vvs)
                    e2 = e2 / xz1
                    ediat[ie, jj, iv - inp.nvini] = e2 / C.conve * C.conve1
                    nobc[ie, jj] = iv
                    ifail = 0
                    ff = np.array(p) / math.sqrt(C.convl)
                    d = splset(ff, r)
                    vals = np.zeros(n1)
                    inside = (r1grid >= r[0]) & (r1grid <= r[NPUNT - 1])
                    vals[inside] = splinqq_many(ff, d, r, r1grid[inside])
                    xnorm = float(np.sum(vals * vals)) * g.ah1
                    fd[ie, jj, iv - inp.nvini] = vals * (math.sqrt(g.ah1) / math.sqrt(xnorm))
            last = nobc[ie, jj] <= 0 if bound_test == "margin" else nobc[ie, jj] == 0
            if last and ifail == -1:
                break                      # no bound levels for higher j
    ediatref = 0.0
    if inp.iprod != 1 and n1 > 1:
        if (inp.nvini <= inp.nvref <= inp.nvmax and inp.jref <= inp.jmax and inp.ielecref <= nelec):
            ediatref = ediat[inp.ielecref - 1, inp.jref - inp.jini, inp.nvref - inp.nvini]
        if inp.no_ref_energy == 0:
            ediatref = 0.0
    return nobc, ediat, fd, ediatref


def product_radialf_write(g, potelebond, nviniprod, nvmaxprod, jiniprod, jmaxprod, n2prod1, r1inf=100.0,
                          nelec=1):
    """Product (02) diatom states on the R grid, the diabatic form of
    product_radialf_write (SRC/mod_baseYfunciones_01y2.f:1065-1308 with
    diabatic_prod_pot > 0): per j, the box DVR of bndbcele
    (SRC/liboctdyn.f:1687-1814) on the npun2 points of [rmis2, rfin2], kinetic
    matrix (-1)^(i-i') (1/(i-i')^2 + 1/(i+i')^2) / (ah^2 mu) off the diagonal
    and (pi^2/6 + 1/(2i)^2) / (ah^2 mu) on it, the lowest nvmaxprod - nviniprod
    + 1 levels kept (all of them, noBCprod = nvmaxprod).  The shipped H + HD run
    took its product states from this form (its log's product levels agree with
    it to 1e-13 eV).  Eigenvector signs are free; each state is made positive
    at its largest component.  Returns (fdprod[njp][nvp][nelec][n2prod1],
    ediatprod[njp][nvp] in zot, nobcprod[njp])."""
    inp = g.inp
    if nelec != 1:
        return _product_dvr_coupled(g, potelebond, nviniprod, nvmaxprod, jiniprod, jmaxprod, n2prod1, r1inf, nelec)
    npun = inp.npun2
    rmis = inp.rmis2 / C.convl
    rfin = inp.rfin2 / C.convl
    ah = (rfin - rmis) / float(npun - 1)
    rg = r1inf / C.convl
    xmu = g.xm1prod * C.convm
    r = rmis + np.arange(npun, dtype=np.float64) * ah
    V = potelebond(np.full(npun, rg), r, 1.0)[0, 0]
    i = np.arange(1, npun + 1)
    menos = (i[:, None] - i[None, :]).astype(np.float64)
    mas = (i[:, None] + i[None, :]).astype(np.float64)
    sign = np.where((i[:, None] - i[None, :]) % 2 == 0, 1.0, -1.0)
    x1 = np.where(menos == 0.0, math.pi * math.pi / 6.0, 1.0 / np.where(menos == 0.0, 1.0, menos * menos))
    T = sign * (x1 + 1.0 / (mas * mas)) / (ah * ah) / xmu
    njp, nvp = jmaxprod - jiniprod + 1, nvmaxprod - nviniprod + 1
    fdprod = np.zeros((njp, nvp, nelec, n2prod1))
    ediatprod = np.zeros((njp, nvp))
    for jj, j in enumerate(range(jiniprod, jmaxprod + 1)):
        xl = 0.5 * float(j * (j + 1)) / xmu
        H = T + np.diag(xl / (r * r) + V)
        w, vec = np.linalg.eigh(H)
        for k, iv in enumerate(range(nviniprod, nvmaxprod + 1)):
            c = vec[:, k]
            if c[np.argmax(np.abs(c))] < 0:
                c = -c
            ediatprod[jj, k] = w[k] / C.conve * C.conve1
            fdprod[jj, k, 0] = (c / math.sqrt(ah))[:n2prod1] * math.sqrt(g.ah2 / C.convl)
    return fdprod, ediatprod, np.full(njp, nvmaxprod, np.int32)


NPUNT_ADIABATIC = 2000


def bndbc1ele(vdiag, xm, rmis, rfin, nvini, nvmax, j, max_viblevels):
    """Bound levels of several uncoupled electronic states for one j
    (SRC/liboctdyn.f:1815-1941): per state the tridiagonal finite-difference
    eigenvalues as guesses, each refined by schr, kept while V(rfin) - E >
    0.01 hartree, up to max_viblevels(state) levels (or nvmax + 2 when it is
    negative), appended state after state (not sorted across states) and
    numbered from nvini - 1.  vdiag [nelec][npun] in hartree, xm in a.u.
    Returns {level: (E hartree, state 1-based, v within the state, function [npun])}
    for the levels numbered nvini..nvmax, and the last level number."""
    nelec, npun = vdiag.shape
    ah = (rfin - rmis) / float(npun - 1)
    xl = 0.5 * float(j * (j + 1)) / xm
    xz, xz1 = 0.5 / xm, 2.0 * xm
    r = rmis + np.arange(npun, dtype=np.float64) * ah
    out = {}
    ivreal = nvini - 1
    for ie in range(nelec):
        vv = vdiag[ie] + xl / (r * r)
        diag = -2.0 - 2.0 * xm * vv * ah * ah
        alpha = np.sort(-xz * eigvalsh_tridiagonal(diag, np.ones(npun - 1)) / ah / ah)
        maxvib = nvmax + 1 if max_viblevels[ie] < 0 else max_viblevels[ie] - 1
        for iv in range(0, min(npun, maxvib) + 1):
            if iv >= npun or not (vdiag[ie, npun - 1] - alpha[iv] > 1.0e-2):
                continue
            e2, _, p = schr(alpha[iv] * xz1, rmis, rfin, npun, 20, 1.0e-10, (vv * xz1).tolist())
            ivreal += 1
            if nvini <= ivreal <= nvmax:
                out[ivreal] = (e2 / xz1, ie + 1, iv, np.array(p))
    return out, ivreal


def product_radialf_write_adiabatic(g, potelebond, nviniprod, nvmaxprod, jiniprod, jmaxprod, n2prod1, r1inf=100.0,
                                    nelec=1, max_viblevels=None):
    """Product (02) diatom states of uncoupled (adiabatic) electronic states,
    the diabatic_prod_pot = 0 branch of product_radialf_write
    (SRC/mod_baseYfunciones_01y2.f:1071-1250): the diagonal potentials of
    potelebond on 2000 points of [rmis2, rfin2] with atom 1 at r1inf, per j
    the levels of bndbc1ele, each level's function (nonzero only in its own
    state) splined onto the first n2prod1 R points and discrete-normalised.
    max_viblevels defaults as the namelist does (-1 per state; nvmaxprod -
    nviniprod + 1 with one state).  Returns (fdprod[njp][nvp][nelec][n2prod1],
    ediatprod[njp][nvp] in zot, nobcprod[njp], elecprodmax[njp][nvp] (the
    level's state), vibelecprod[njp][nvp] (its v within the state))."""
    inp = g.inp
    if max_viblevels is None:
        max_viblevels = [nvmaxprod - nviniprod + 1] if nelec == 1 else [-1] * nelec
    npunt = NPUNT_ADIABATIC
    rmis, rfin = inp.rmis2 / C.convl, inp.rfin2 / C.convl
    ah = (rfin - rmis) / float(npunt - 1)
    r = rmis + np.arange(npunt, dtype=np.float64) * ah
    V = potelebond(np.full(npunt, r1inf / C.convl), r, 1.0)
    vdiag = np.array([V[ie, ie] for ie in range(nelec)])
    xm = g.xm1prod * C.convm
    njp, nvp = jmaxprod - jiniprod + 1, nvmaxprod - nviniprod + 1
    fdprod = np.zeros((njp, nvp, nelec, n2prod1))
    ediatprod = np.zeros((njp, nvp))
    nobcprod = np.full(njp, nviniprod - 1, np.int32)
    elecprodmax = np.zeros((njp, nvp), np.int32)
    vibelecprod = np.zeros((njp, nvp), np.int32)
    r2 = (inp.rmis2 + np.arange(n2prod1, dtype=np.float64) * g.ah2) / C.convl
    inside = (r2 >= r[0]) & (r2 <= r[-1])
    for jj, j in enumerate(range(jiniprod, jmaxprod + 1)):
        levels, ivreal = bndbc1ele(vdiag, xm, rmis, rfin, nviniprod, nvmaxprod, j, max_viblevels)
        for iv in range(nviniprod, min(ivreal, nvmaxprod) + 1):
            e, ie, v, p = levels[iv]
            k = iv - nviniprod
            ediatprod[jj, k] = e / C.conve * C.conve1
            ff = p / math.sqrt(C.convl)
            d = splset(ff, r)
            vals = np.zeros(n2prod1)
            vals[inside] = splinqq_many(ff, d, r, r2[inside])
            xnorm = float(np.sum(vals * vals)) * g.ah2
            if xnorm > 1.0e-8:
                vals = vals * math.sqrt(g.ah2 / xnorm)
            fdprod[jj, k, ie - 1] = vals
            elecprodmax[jj, k] = ie
            vibelecprod[jj, k] = v
        nobcprod[jj] = min(ivreal, nvmaxprod)
    return fdprod, ediatprod, nobcprod, elecprodmax, vibelecprod


def _dvr_kinetic(npun, ah, xmu):
    """bndbcele's particle-in-a-box DVR kinetic matrix (SRC/liboctdyn.f:1760-1779)."""
    i = np.arange(1, npun + 1)
    menos = (i[:, None] - i[None, :]).astype(np.float64)
    mas = (i[:, None] + i[None, :]).astype(np.float64)
    sign = np.where((i[:, None] - i[None, :]) % 2 == 0, 1.0, -1.0)
    x1 = np.where(menos == 0.0, math.pi * math.pi / 6.0, 1.0 / np.where(menos == 0.0, 1.0, menos * menos))
    return sign * (x1 + 1.0 / (mas * mas)) / (ah * ah) / xmu


def _product_dvr_coupled(g, potelebond, nviniprod, nvmaxprod, jiniprod, jmaxprod, n2prod1, r1inf, nelec):
    """product_radialf_write's diabatic branch for several coupled states
    (bndbcele, SRC/liboctdyn.f:1687-1814): one block per state holding the DVR
    kinetic matrix and the centrifugal term, the potential matrix coupling the
    states at each point; the lowest nvmaxprod - nviniprod + 1 levels, each
    eigenvector positive at its largest component, its state components
    discrete-normalised as one vector over the npun2 points."""
    inp = g.inp
    npun = inp.npun2
    rmis, rfin = inp.rmis2 / C.convl, inp.rfin2 / C.convl
    ah = (rfin - rmis) / float(npun - 1)
    xmu = g.xm1prod * C.convm
    r = rmis + np.arange(npun, dtype=np.float64) * ah
    V = potelebond(np.full(npun, r1inf / C.convl), r, 1.0)
    T = _dvr_kinetic(npun, ah, xmu)
    njp, nvp = jmaxprod - jiniprod + 1, nvmaxprod - nviniprod + 1
    fdprod = np.zeros((njp, nvp, nelec, n2prod1))
    ediatprod = np.zeros((njp, nvp))
    for jj, j in enumerate(range(jiniprod, jmaxprod + 1)):
        xl = 0.5 * float(j * (j + 1)) / xmu
        H = np.zeros((nelec * npun, nelec * npun))
        for e in range(nelec):
            H[e * npun:(e + 1) * npun, e * npun:(e + 1) * npun] = T + np.diag(xl / (r * r))
            for f in range(nelec):
                H[e * npun:(e + 1) * npun, f * npun:(f + 1) * npun] += np.diag(V[e, f])
        w, vec = np.linalg.eigh(H)
        for k in range(nvp):
            c = vec[:, k]
            if c[np.argmax(np.abs(c))] < 0:
                c = -c
            ediatprod[jj, k] = w[k] / C.conve * C.conve1
            fdprod[jj, k] = (c.reshape(nelec, npun) / math.sqrt(ah))[:, :n2prod1] * math.sqrt(g.ah2 / C.convl)
    return fdprod, ediatprod, np.full(njp, nvmaxprod, np.int32)


def product_labels(fdprod, nviniprod):
    """elecprodmax and vibelecprod of diabatic product states
    (SRC/mod_baseYfunciones_01y2.f:1190-1245): the state holding the largest
    share of each level's norm (the first on ties), and the level number itself."""
    njp, nvp = fdprod.shape[:2]
    norms = np.sum(fdprod ** 2, axis=3)                     # [njp][nvp][nelec]
    elec = np.argmax(norms, axis=2).astype(np.int32) + 1
    vib = np.broadcast_to(nviniprod + np.arange(nvp, dtype=np.int32), (njp, nvp)).copy()
    return elec, vib


def write_func(outdir, inp, nobc, ediat, fd, ediatref, nelec=1):
    """func/bcwf and func/eref (SRC/mod_baseYfunciones_01y2.f:785-808)."""
    os.makedirs(os.path.join(outdir, "func"), exist_ok=True)
    lines = []
    for ie in range(nelec):
        for jj, j in enumerate(range(inp.jini, inp.jmax + 1)):
            lines.append("%d %d %d" % (ie + 1, j, nobc[ie, jj]))
            for iv in range(inp.nvini, nobc[ie, jj] + 1):
                lines.append("%d %r" % (iv, float(ediat[ie, jj, iv - inp.nvini])))
                lines.extend(repr(float(x)) for x in fd[ie, jj, iv - inp.nvini])
    with open(os.path.join(outdir, "func", "bcwf"), "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(os.path.join(outdir, "func", "eref"), "w") as f:
        f.write("%r\n" % float(ediatref))


def write_prodwf(outdir, jiniprod, nviniprod, fdprod, ediatprod, nobcprod, elecprodmax=None, vibelecprod=None):
    """func/prodwf (SRC/mod_baseYfunciones_01y2.f:1267-1281): per product j the
    line 'j noBCprod(j) n2prod1 nelec', then per v in nviniprod..noBCprod(j)
    the line 'v E(v,j) elecprodmax vibelecprod' (E in zot, unshifted) and
    n2prod1 lines of fdprod(ir2, v, j, 1..nelec).  fdprod is
    [njp][nvp][nelec][n2prod1], ediatprod [njp][nvp]; elecprodmax and
    vibelecprod default to state 1 and v itself (diabatic products)."""
    os.makedirs(os.path.join(outdir, "func"), exist_ok=True)
    njp, nvp, nelec, n2p = fdprod.shape
    lines = []
    for jj in range(njp):
        nob = int(nobcprod[jj])
        lines.append("%d %d %d %d" % (jiniprod + jj, nob, n2p, nelec))
        for iv in range(nviniprod, nob + 1):
            k = iv - nviniprod
            em = 1 if elecprodmax is None else int(elecprodmax[jj, k])
            vb = iv if vibelecprod is None else int(vibelecprod[jj, k])
            lines.append("%d %r %d %d" % (iv, float(ediatprod[jj, k]), em, vb))
            for ir2 in range(n2p):
                lines.append(" ".join(repr(float(fdprod[jj, k, e, ir2])) for e in range(nelec)))
    with open(os.path.join(outdir, "func", "prodwf"), "w") as f:
        f.write("\n".join(lines) + "\n")


def pot1(g, potelebond, vref, outdir, nelec=1, states=None):
    """SRC/mod_pot_01y2.f:147-341 for one electronic state: V on the grid in
    zot minus vref, stored where it lies below Vcut (capped at Vcut otherwise);
    pot/pot.NNN.dat rows 'ir1 ir2 V' with ir2 outer and ir1 inner, and
    pot/cont.pot.  Several states: see _pot1_coupled (``states``: per state
    (iomdiat, iomatom, sigdiat, sigatom) for cont.pot, default (0, 0, 1, 1)).
    Returns (npunreal, vmin, vmaxtot)."""
    if nelec != 1:
        return _pot1_coupled(g, potelebond, vref, outdir, nelec, states)
    inp = g.inp
    os.makedirs(os.path.join(outdir, "pot"), exist_ok=True)
    n1, n2 = inp.npun1, inp.npun2
    vcut = g.vcutmax
    r1 = inp.rmis1 + np.arange(n1, dtype=np.float64) * g.ah1
    r2 = inp.rmis2 + np.arange(n2, dtype=np.float64) * g.ah2
    rpeq = np.broadcast_to((r1 / C.convl)[None, :], (n2, n1))     # [ir2][ir1]
    Rg = np.broadcast_to((r2 / C.convl)[:, None], (n2, n1))
    gam = inp.xm1 / (inp.xm0 + inp.xm1)
    vmin = 1e10
    vmaxtot = vcut
    npunreal = []
    for iang in range(inp.nangu):
        ctet = float(g.cgamma[iang])
        X2 = np.sqrt(Rg * Rg + gam * gam * rpeq * rpeq + 2.0 * gam * Rg * rpeq * ctet)
        calpha = (Rg * ctet + gam * rpeq) / X2
        calpha = np.where(np.abs(calpha) > 1.0, calpha / np.abs(calpha), calpha)
        with np.errstate(invalid="ignore"):
            pm = potelebond(rpeq, X2, calpha)[0, 0]
        v = pm / C.conve * C.conve1 - vref
        v = np.where(v > vcut, vcut, v)
        vmaxtot = max(vmaxtot, float(np.nanmax(v)))
        vmin = min(vmin, float(np.nanmin(v)))
        keep = v < vcut
        i2, i1 = np.nonzero(keep)
        vals = v[i2, i1]
        with open(os.path.join(outdir, "pot", "pot.%03d.dat" % (iang + 1)), "w") as f:
            f.write("".join("%d %d %r\n" % (a + 1, b + 1, float(x)) for a, b, x in zip(i1, i2, vals)))
        npunreal.append(len(i1))
    with open(os.path.join(outdir, "pot", "cont.pot"), "w") as f:
        f.write("%d\n0 0 1.0 1.0\n" % nelec)
        f.write("%r %d %r\n" % (vmin, sum(npunreal), vmaxtot))
        f.write("%r %r %d\n" % (inp.rmis1, inp.rfin1, n1))
        f.write("%r %r %d\n" % (inp.rmis2, inp.rfin2, n2))
        f.write("%d %d\n" % (inp.nangu, inp.inc))
        f.write(" ".join("%d" % n for n in npunreal) + "\n")
    return np.array(npunreal, np.int32), vmin, vmaxtot


def _pot1_coupled(g, potelebond, vref, outdir, nelec, states=None):
    """pot1 for several electronic states (SRC/mod_pot_01y2.f:147-341): at each
    grid point the potential matrix in zot with vref subtracted on the
    diagonal; a state whose diagonal exceeds Vcut has its row and
    column zeroed and the diagonal set to Vcut (in state order); the point is
    stored when any eigenvalue of the matrix lies below Vcut, as 'ir1 ir2'
    and the matrix column by column; vmin and vmaxtot are the extreme
    eigenvalues over the grid (vmaxtot at least Vcut)."""
    inp = g.inp
    os.makedirs(os.path.join(outdir, "pot"), exist_ok=True)
    n1, n2 = inp.npun1, inp.npun2
    vcut = g.vcutmax
    states = states or [(0, 0, 1.0, 1.0)] * nelec
    r1 = inp.rmis1 + np.arange(n1, dtype=np.float64) * g.ah1
    r2 = inp.rmis2 + np.arange(n2, dtype=np.float64) * g.ah2
    rpeq = np.broadcast_to((r1 / C.convl)[None, :], (n2, n1))     # [ir2][ir1]
    Rg = np.broadcast_to((r2 / C.convl)[:, None], (n2, n1))
    gam = inp.xm1 / (inp.xm0 + inp.xm1)
    vmin, vmaxtot = 1e10, vcut
    npunreal = []
    for iang in range(inp.nangu):
        ctet = float(g.cgamma[iang])
        X2 = np.sqrt(Rg * Rg + gam * gam * rpeq * rpeq + 2.0 * gam * Rg * rpeq * ctet)
        calpha = (Rg * ctet + gam * rpeq) / X2
        calpha = np.where(np.abs(calpha) > 1.0, calpha / np.abs(calpha), calpha)
        with np.errstate(invalid="ignore"):
            v = potelebond(rpeq, X2, calpha) / C.conve * C.conve1     # [ne][ne][n2][n1]
        v = np.array(v, dtype=np.float64)
        for e in range(nelec):
            v[e, e] -= vref
        for e in range(nelec):
            hi = v[e, e] > vcut
            for f in range(nelec):
                v[e, f] = np.where(hi, 0.0, v[e, f])
                v[f, e] = np.where(hi, 0.0, v[f, e])
            v[e, e] = np.where(hi, vcut, v[e, e])
        eig = np.moveaxis(np.linalg.eigvalsh(np.moveaxis(v, (0, 1), (-2, -1))), -1, 0)   # [ne][n2][n1]
        vmaxtot = max(vmaxtot, float(np.nanmax(eig)))
        vmin = min(vmin, float(np.nanmin(eig)))
        keep = (eig < vcut).any(axis=0)
        i2, i1 = np.nonzero(keep)
        with open(os.path.join(outdir, "pot", "pot.%03d.dat" % (iang + 1)), "w") as f:
            for a, b in zip(i1, i2):
                vals = [float(v[ie, je, b, a]) for je in range(nelec) for ie in range(nelec)]
                f.write("%d %d %s\n" % (a + 1, b + 1, " ".join(repr(x) for x in vals)))
        npunreal.append(len(i1))
    with open(os.path.join(outdir, "pot", "cont.pot"), "w") as f:
        f.write("%d\n" % nelec)
        for st in states:
            f.write("%d %d %r %r\n" % (int(st[0]), int(st[1]), float(st[2]), float(st[3])))
        f.write("%r %d %r\n" % (vmin, sum(npunreal), vmaxtot))
        f.write("%r %r %d\n" % (inp.rmis1, inp.rfin1, n1))
        f.write("%r %r %d\n" % (inp.rmis2, inp.rfin2, n2))
        f.write("%d %d\n" % (inp.nangu, inp.inc))
        f.write(" ".join("%d" % n for n in npunreal) + "\n")
    return np.array(npunreal, np.int32), vmin, vmaxtot


def write_case(outdir, inputfile, potelebond, bound_test="margin", input_text=None, product_form="dvr",
               states=None):
    """pot.out for one input.dat (a path, or its text in ``input_text``) and a
    surface: func/ and pot/ beside a copy of the input, for the input's
    nelecmax states (``states``: their (iomdiat, iomatom, sigdiat, sigatom)).
    With iprod = 2 the product states are written to func/prodwf:
    ``product_form`` "dvr" takes the box DVR of bndbcele (the form the shipped
    H + HD run was made with), "namelist" follows &inputpotmass's
    diabatic_prod_pot as the current source does (0, its default: the
    uncoupled-state levels of bndbc1ele).  Returns a summary (levels, eref,
    points per angle, vmin, product states)."""
    groups = namelist.parse(input_text) if input_text is not None else namelist.read(inputfile)
    inp, flat = _inputs(groups)
    nelec = int(inp.nelecmax)
    os.makedirs(outdir, exist_ok=True)
    with open(os.path.join(outdir, "input.dat"), "w") as f:
        f.write(namelist.dumps(groups))
    g = _grid(inp)
    r2inf = float(flat.get("r2inf_radial_functions", 100.0))
    nobc, ediat, fd, eref = radial_functions01_write(g, potelebond, r2inf=r2inf, nelec=nelec,
                                                     bound_test=bound_test)
    write_func(outdir, inp, nobc, ediat, fd, eref, nelec=nelec)
    npunreal, vmin, vmaxtot = pot1(g, potelebond, eref, outdir, nelec=nelec, states=states)
    out = {"nobc": nobc, "ediat": ediat, "fd": fd, "ediatref": eref, "npunreal": npunreal,
           "vmin": vmin, "vmaxtot": vmaxtot, "cgamma": g.cgamma}
    prod = groups.get("inputprod", {})
    if int(prod.get("iprod", 0)) == 2:
        nv0, nv1 = int(prod.get("nviniprod", 0)), int(prod.get("nvmaxprod", 0))
        j0, j1 = int(prod.get("jiniprod", 0)), int(prod.get("jmaxprod", 0))
        n2p = int(prod.get("n2prod1", inp.npun2))
        r1inf = float(flat.get("r1inf_radial_functions", 100.0))
        dia = int(groups.get("inputpotmass", {}).get("diabatic_prod_pot", 0))
        if product_form == "dvr" or (product_form == "namelist" and dia > 0):
            fdp, edp, nobp = product_radialf_write(g, potelebond, nv0, nv1, j0, j1, n2p, r1inf=r1inf, nelec=nelec)
            elec, vib = product_labels(fdp, nv0)
            out["product"] = (fdp, edp, nobp)
        elif product_form == "namelist":
            mv = prod.get("max_viblevels")
            mv = None if mv is None else list(np.atleast_1d(mv).astype(int))
            fdp, edp, nobp, elec, vib = product_radialf_write_adiabatic(g, potelebond, nv0, nv1, j0, j1, n2p,
                                                                        r1inf=r1inf, nelec=nelec, max_viblevels=mv)
            out["product"] = (fdp, edp, nobp)
        else:
            raise ValueError("product_form must be 'dvr' or 'namelist'")
        write_prodwf(outdir, j0, nv0, fdp, edp, nobp, elec, vib)
    return out
