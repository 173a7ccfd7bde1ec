"""Bound states on the propagation grid by Lanczos: the host side of the
reference's bndgrid.out (SRC/bound-lanz/main_boundlanz.f), the second caller
of the H psi boundary besides the Chebyshev loop.

The reference evaluates H phi through Hmatrix (main_boundlanz.f:332-357),
which copies phi into the propagation vector, calls difs and copies H phi
back; here the operator is any callable psi -> H psi on the wave's state
vector layout, normally ``Propagator(run, "fp64").hphi`` (mw3_hphi, host
arrays in and out, like Hmatrix).  The algorithms follow
SRC/bound-lanz/liboctdynlanz.f:

* ``lanczos_eigenvalues``: lanzvalpariter (:3-278), the non-orthogonal Lanczos
  recursion of Cullum and Willoughby, with the converged eigenvalues taken
  every ``ntimes`` steps by ``converged_eigenvalues`` (valnkry, :472-575):
  eigenvalues of the tridiagonal T and of T with its first row and column
  removed; multiple copies are true, simple ones are true unless T-hat has
  them too (spurious), both to 1e-8 zot.
* ``cg_eigenvector``: cgradvecpar (:280-470), the eigenvector of a converged
  eigenvalue by conjugate gradients on H - E from the initial guess.
* ``initial_vector``: initia_lanzvec (main_boundlanz.f:270-330), a flat vector
  on the stored points whose diagonal potential lies below Emax_lanzini.

The tridiagonal eigenvalues come from LAPACK (scipy's eigh_tridiagonal)
instead of the reference's QL routine (TQLI, SRC/liboctdyn.f:233-289); both are
backward stable, so the eigenvalues agree to rounding, far inside the 1e-8
zot that separates true from spurious copies.  State assignment (bndassign)
and the plotting of the states need the product-channel functions and are
not part of this module.
"""
import math

import numpy as np

from .host.constants import conve1, eV2cm, ev_to_zot

GHOST_TOL = 1.0e-8          # zot; valnkry's critener


def initial_vector(run, emax_zot):
    """initia_lanzvec (main_boundlanz.f:270-330): 1 on every stored point whose
    diagonal potential V(ir, iang, e, e) of its block's electronic state is
    below emax_zot, 0 elsewhere, normalised.  Raises if no point qualifies (the
    reference stops with 'Norm too low')."""
    blk, ang, _, _ = run.point_table()
    ir = np.empty(run.ntot, np.int64)
    for iang in run.angle_order():
        n = run.npunreal[iang - 1]
        for b in range(run.ncan):
            o = run.offs[iang - 1, b]
            ir[o:o + n] = np.arange(n)
    ele = np.asarray(run.nelebas)[blk] - 1
    v = run.vvv[ele, ele, ang - 1, ir]
    x = np.where(v < emax_zot, 1.0, 0.0)
    nrm = float(np.dot(x, x))
    if abs(nrm) < 1e-10:
        raise ValueError("initial Lanczos vector has no point below Emax_lanzini (norm too low)")
    return x / np.sqrt(nrm)


def converged_eigenvalues(alpha, beta, tol=GHOST_TOL):
    """valnkry (liboctdynlanz.f:472-575).  alpha[0..n-1] is the diagonal of the
    Lanczos matrix T, beta[i] couples i and i+1 (beta[n-1], if given, is not
    used).  Returns the sorted eigenvalues accepted as true."""
    from scipy.linalg import eigh_tridiagonal

    a = np.asarray(alpha, np.float64)
    n = a.size
    if n == 0:
        return np.zeros(0)
    b = np.asarray(beta, np.float64)[:n - 1]
    ev = np.sort(eigh_tridiagonal(a, b, eigvals_only=True)) if n > 1 else a.copy()
    # T-hat: first row and column decoupled (betar(1) = 0)
    if n > 2:
        evr = np.sort(np.concatenate([[a[0]], eigh_tridiagonal(a[1:], b[1:], eigvals_only=True)]))
    else:
        evr = np.sort(a.copy())
    # group the sorted eigenvalues: a value within tol of its group's first joins it
    groups = []                 # [first value, copies]
    for e in ev:
        if groups and abs(groups[-1][0] - e) < tol:
            groups[-1][1] += 1
        else:
            groups.append([e, 1])
    out = []
    for e, deg in groups:
        if deg > 1:
            out.append(e)
        elif not np.any(np.abs(evr - e) < tol):
            out.append(e)
    return np.asarray(out)


def lanczos_eigenvalues(hphi, v1, nkrymax=10000, ntimes=1000, on_block=None):
    """lanzvalpariter (liboctdynlanz.f:3-278) from the normalised start vector v1.

    The recursion runs in blocks of ``ntimes`` steps; after each block the
    converged eigenvalues of the Krylov matrix so far are computed (and passed
    to ``on_block(nkry, etrue)`` if given).  As in the reference the loop ends
    once the Krylov dimension reaches nkrymax - 1 or more, so the last block
    can take it to nkrymax + 1.  Returns (etrue, alpha, beta)."""
    if ntimes < 2:
        raise ValueError("ntimes must be at least 2")
    v1 = np.ascontiguousarray(v1, np.float64)
    alpha, beta = [], []
    f2 = v1                                   # flanz(:,2)
    hu = hphi(f2)
    alpha.append(float(np.dot(hu, f2)))
    f1 = hu - alpha[0] * f2
    beta.append(float(np.sqrt(np.dot(f1, f1))))
    f1 = f1 / beta[0]
    hu = hphi(f1)
    alpha.append(float(np.dot(hu, f1) - beta[0] * np.dot(f2, f1)))
    nkry = 2                                  # alpha(1), alpha(2) known
    etrue = np.zeros(0)
    first = True
    while True:
        target = (1 + ntimes) if first else nkry + ntimes
        first = False
        while nkry < target:
            f0 = hu - alpha[nkry - 1] * f1 - beta[nkry - 2] * f2
            b = float(np.sqrt(np.dot(f0, f0)))
            if len(beta) < nkry:
                beta.append(b)
            else:
                beta[nkry - 1] = b
            f0 = f0 / b
            hu = hphi(f0)
            alpha.append(float(np.dot(hu, f0) - b * np.dot(f1, f0)))
            f2, f1 = f1, f0
            nkry += 1
        # beta(nkry): the norm of the next residual
        x = hu - alpha[nkry - 1] * f1 - beta[nkry - 2] * f2
        b = float(np.sqrt(np.dot(x, x)))
        if len(beta) < nkry:
            beta.append(b)
        else:
            beta[nkry - 1] = b
        etrue = converged_eigenvalues(alpha[:nkry], beta[:nkry])
        if on_block is not None:
            on_block(nkry, etrue)
        if nkry + 1 >= nkrymax:
            break
    return etrue, np.asarray(alpha), np.asarray(beta)


def cg_eigenvector(hphi, v0, ediag, nomxiter, criter):
    """cgradvecpar (liboctdynlanz.f:280-470): conjugate gradients on A = H - ediag
    from v0, renormalising v every step, until the mean energy <v|H|v> is
    within criter of ediag or nomxiter steps are done.  Returns
    (v, emean, iterations, converged)."""
    v = np.array(v0, np.float64)

    def a_op(x):
        return hphi(x) - ediag * x

    r = a_op(v)
    p = -r
    ap = a_op(p)
    lam = -float(np.dot(r, p)) / float(np.dot(p, ap))
    it = 0
    emean = ediag
    while True:
        it += 1
        v = v + lam * p
        v = v / np.sqrt(float(np.dot(v, v)))
        hv = hphi(v)
        emean = float(np.dot(hv, v))
        r = hv - ediag * v
        ap = a_op(p)
        eps = float(np.dot(r, ap)) / float(np.dot(p, ap))
        p = eps * p - r
        ap = a_op(p)
        lam = -float(np.dot(r, p)) / float(np.dot(p, ap))
        if it > nomxiter:
            return v, emean, it, False
        if abs(emean - ediag) <= criter:
            return v, emean, it, True


def write_levels(path, etrue, vcutmax):
    """niveles.dat (main_boundlanz.f:186-200): index, zot, cm^-1 and eV of
    every converged eigenvalue below vcutmax, format (1x,i5,3(2x,e15.7))."""
    with open(path, "w") as f:
        for i, e in enumerate(etrue, 1):
            if e < vcutmax:
                f.write(" %5d  %s  %s  %s\n" % (i, _e15(e), _e15(e / conve1), _e15(e / conve1 / eV2cm)))


def _e15(x):
    """Fortran e15.7."""
    from .printprob import fortran_e
    return fortran_e(x, 15, 7, 2)


def _point_labels(run):
    """Per flat point: (icanp, ielec, iom, iangp, ir, ir1, ir2, iang), 1-based as
    indiproc gives them for one process (SRC/mod_pot_01y2.f:628-654)."""
    order = list(run.angle_order())
    rows = np.zeros((run.ntot, 8), np.int64)
    for iangp, iang in enumerate(order, 1):
        n = run.npunreal[iang - 1]
        for b in range(run.ncan):
            o = run.offs[iang - 1, b]
            rows[o:o + n, 0] = b + 1
            rows[o:o + n, 1] = run.nelebas[b]
            rows[o:o + n, 2] = run.iombas[b]
            rows[o:o + n, 3] = iangp
            rows[o:o + n, 4] = np.arange(1, n + 1)
            rows[o:o + n, 5] = run.indr1[iang - 1, :n]
            rows[o:o + n, 6] = run.indr2[iang - 1, :n]
            rows[o:o + n, 7] = iang
    return rows


def write_bnd(outdir, run, iv, energy_zot, vec, idproc=0):
    """write_bnd (main_boundlanz.f:360-400): bnd.ivNNN.ipNNN (iv, E in eV, then
    the vector one value per line) and grid.ipNNN (the grid and every point's
    indices, (9(1x,i7)))."""
    import os
    lab = _point_labels(run)
    i = run.inp
    with open(os.path.join(outdir, "bnd.iv%03d.ip%03d" % (iv, idproc)), "w") as f:
        f.write(" %d %r\n" % (iv, float(energy_zot) / conve1 / eV2cm))
        f.writelines(" %r\n" % float(x) for x in vec)
    with open(os.path.join(outdir, "grid.ip%03d" % idproc), "w") as f:
        f.write(" %d\n" % run.ntot)
        f.write(" %r %r %d\n" % (float(i.rmis1), float(i.rfin1), i.npun1))
        f.write(" %r %r %d\n" % (float(i.rmis2), float(i.rfin2), i.npun2))
        f.write(" %d %d\n" % (i.nangu, i.inc))
        for k in range(run.ntot):
            f.write("".join(" %7d" % x for x in (k + 1,) + tuple(lab[k])) + "\n")


def plot_bnd(outdir, run, iv, vec):
    """plot_bnd (main_boundlanz.f:620-811), three plot files of a bound state
    (lines '(100(1x,e15.7))', a blank line after each block):
      bndplot.iNNN     R, gamma (radians), sum over r1 and channels of psi^2, per R;
      bndr1r2.iNNN     r1, R, sum over angles and channels of psi^2, per R;
      bndbondx1x2.iNNN x1, x2, psi along the cut at a 135.5 degree bond angle, per x1:
    for r1 = x1 and a second bond x2 on the r1 grid, R = (x2^2 + g^2 x1^2 -
    2 cos(135.5) g x1 x2)^(1/2) with g = m1/(m0+m1), taken at the R index
    INT((R - rmis2)/ah2) (the program's truncation, clamped to the grid) and at
    the first angle whose cos gamma is nearest (x2 cos(135.5) - g x1)/R; the
    value is psi (not squared) of the last stored point there in flat order, 0
    where none is stored."""
    import os
    i = run.inp
    na, n1, n2 = i.nangu, i.npun1, i.npun2
    lab = _point_labels(run)
    ir1, ir2, iang = lab[:, 5] - 1, lab[:, 6] - 1, lab[:, 7] - 1
    vec = np.asarray(vec, np.float64)
    p2 = vec * vec
    cg = np.asarray(run.cgamma[:na], np.float64)
    line = lambda vals: "".join(" " + _e15(v) for v in vals) + "\n"
    by_ang = np.zeros((n2, na))
    np.add.at(by_ang, (ir2, iang), p2)
    with open(os.path.join(outdir, "bndplot.i%03d" % iv), "w") as f:
        for jr2 in range(n2):
            r2 = i.rmis2 + jr2 * run.ah2
            for a in range(na):
                f.write(line((r2, math.acos(cg[a]), by_ang[jr2, a])))
            f.write("\n")
    by_r1 = np.zeros((n2, n1))
    np.add.at(by_r1, (ir2, ir1), p2)
    with open(os.path.join(outdir, "bndr1r2.i%03d" % iv), "w") as f:
        for jr2 in range(n2):
            r2 = i.rmis2 + jr2 * run.ah2
            for k in range(n1):
                f.write(line((i.rmis1 + k * run.ah1, r2, by_r1[jr2, k])))
            f.write("\n")
    last = {}
    for k in range(run.ntot):                  # later points overwrite earlier ones
        last[(ir1[k], ir2[k], iang[k])] = vec[k]
    xb = math.cos(135.5 * math.pi / 180.0)
    gam = i.xm1 / (i.xm0 + i.xm1)
    with open(os.path.join(outdir, "bndbondx1x2.i%03d" % iv), "w") as f:
        for jr1 in range(n1):
            x1 = i.rmis1 + jr1 * run.ah1
            for jr2 in range(n1):
                x2 = i.rmis1 + jr2 * run.ah1
                rg = math.sqrt(x2 * x2 + x1 * x1 * gam * gam - 2.0 * xb * gam * x1 * x2)
                k2 = min(max(int((rg - i.rmis2) / run.ah2), 1), n2)
                ct = (x2 * xb - gam * x1) / rg
                if abs(ct) > 1.0:
                    ct = ct / abs(ct)
                dis, ka = 1.0e10, 0
                for a in range(na):
                    d = abs(cg[a] - ct) ** 2
                    if d < dis:
                        dis, ka = d, a
                f.write(line((x1, x2, last.get((jr1, k2 - 1, ka), 0.0))))
            f.write("\n")


def read_bound_state(run, outdir, iv, idproc=0):
    """A bound state write_bnd stored (bnd.ivNNN.ipNNN, grid.ipNNN), checked to
    lie on the run's grid as dip_bndgrid checks it (SRC/mod_photoini_01y2.f:
    537-650).  Returns ({(ir1, ir2, iang, Omega, ielec): value}, (nr1, nr2,
    nang, Omega max, electronic states), energy in eV)."""
    import os
    i = run.inp
    with open(os.path.join(outdir, "grid.ip%03d" % idproc)) as f:
        n = int(f.readline())
        r1 = f.readline().split()
        r2 = f.readline().split()
        na, inc = (int(x) for x in f.readline().split())
        ah1b = (float(r1[1]) - float(r1[0])) / (int(r1[2]) - 1)
        ah2b = (float(r2[1]) - float(r2[0])) / (int(r2[2]) - 1)
        if abs(i.rmis1 - float(r1[0])) > 1e-4 or abs(run.ah1 - ah1b) > 1e-4 or \
                abs(i.rmis2 - float(r2[0])) > 1e-4 or abs(run.ah2 - ah2b) > 1e-4 or na != i.nangu or inc != i.inc:
            raise ValueError("the bound state was computed on another grid")
        lab = np.array([[int(x) for x in f.readline().split()] for _ in range(n)])
    with open(os.path.join(outdir, "bnd.iv%03d.ip%03d" % (iv, idproc))) as f:
        e_ev = float(f.readline().split()[1])
        val = np.array([float(f.readline()) for _ in range(n)])
    key = {}
    # columns: i, icanp, ielec, iom, iangp, ir, ir1, ir2, iang
    for row, x in zip(lab, val):
        key[(row[6], row[7], row[8], row[3], row[2])] = x     # ir1, ir2, iang, iom, ielec
    dims = (lab[:, 6].max(), lab[:, 7].max(), lab[:, 8].max(), lab[:, 3].max(), lab[:, 2].max())
    return key, dims, e_ev


def initial_from_bound(run, outdir, iv, nelec_bnd=None, idproc=0):
    """dip_bndgrid for iphoto = 2 (SRC/mod_photoini_01y2.f:509-717): the initial
    packet from a bound state that write_bnd stored on the same radial and
    angular grid, point by point through (ir1, ir2, gamma, Omega, electronic
    state); points of the run outside the stored state's range stay 0.
    Returns (psi0, energy in eV, norm of the mapped part).  The dipole-weighted
    form (iphoto = 1) is madwave3_gb300.photo.initial_packet."""
    key, (nr1, nr2, nang, omax, nel0), e_ev = read_bound_state(run, outdir, iv, idproc)
    nel = nel0 if nelec_bnd is None else nelec_bnd
    me = _point_labels(run)
    psi0 = np.zeros(run.ntot)
    for k in range(run.ntot):
        icanp, ielec, iom, iangp, ir, ir1, ir2, iang = me[k]
        if ir1 <= nr1 and ir2 <= nr2 and iang <= nang and iom <= omax and ielec <= nel:
            psi0[k] = key.get((ir1, ir2, iang, iom, ielec), 0.0)
    return psi0, e_ev, float(np.dot(psi0, psi0))


def assign(run, vec, fdprod=None, nviniprod=0):
    """bndassign (main_boundlanz.f:437-617): the distributions that label a
    bound state.  disv1[v] = sum over blocks and (angle, R) of (sum over r1 of
    fd(r1, v, j=0, e) psi)^2 with the reactant diatom's functions; disv2[v'] the
    same over R with the product diatom's (fdprod[nvp][nelec][n2prod1] at
    j' = 0, from ``generator.product_states`` or the host's own), when given;
    <cos gamma>; the populations of every Omega and electronic state."""
    i = run.inp
    lab = _point_labels(run)
    blk, ele, iom, ir1, ir2, iang = (lab[:, 0] - 1, lab[:, 1] - 1, lab[:, 2], lab[:, 5] - 1, lab[:, 6] - 1,
                                     lab[:, 7] - 1)
    v = np.asarray(vec, np.float64)
    nv = i.nvmax - i.nvini + 1
    if i.jini != 0:
        raise ValueError("bndassign projects on j = 0: needs jini = 0")
    key = (blk * i.nangu + iang) * i.npun2 + ir2                 # (block, angle, R) line of each point
    disv1 = np.zeros(nv)
    for k in range(nv):
        w = run.fd[ele, 0, k, ir1] * v
        disv1[k] = np.sum(np.bincount(key, weights=w) ** 2)
    disv2 = None
    if fdprod is not None:
        fdprod = np.asarray(fdprod)
        n2p = fdprod.shape[-1]
        key2 = (blk * i.nangu + iang) * i.npun1 + ir1            # (block, angle, r1) line
        inside = ir2 < n2p
        disv2 = np.zeros(fdprod.shape[0])
        for k in range(fdprod.shape[0]):
            w = np.where(inside, fdprod[k, ele, np.minimum(ir2, n2p - 1)], 0.0) * v
            disv2[k] = np.sum(np.bincount(key2, weights=w) ** 2)
    cos_mean = float(np.sum(v * v * run.cgamma[iang]))
    disomg = {int(o): float(np.sum(v[iom == o] ** 2)) for o in range(i.iommin, i.iommax + 1)}
    diselec = np.array([np.sum(v[ele == e] ** 2) for e in range(run.nelec)])
    return dict(disv1=disv1, disv2=disv2, cos_mean=cos_mean, disomg=disomg, diselec=diselec)


class BoundStates:
    """bndgrid.out's Lanczos part for one wave: eigenvalues, then eigenvectors of
    the lowest ones.  Parameters are the reference's &lanczos_parameters
    (mod_lanczos_01y2.f:31-55, defaults as there), energies in eV."""

    def __init__(self, run, hphi, emax_lanzini_ev, ntimes=1000, nkrymax=10000, criter_ev=1e-4,
                 nomxiter=None, nvecmin=1, nvecmax=10):
        self.run = run
        self.hphi = hphi
        self.emax = ev_to_zot(emax_lanzini_ev)
        self.ntimes = ntimes
        self.nkrymax = nkrymax
        self.criter = ev_to_zot(criter_ev)
        self.nomxiter = nkrymax if nomxiter is None else nomxiter
        self.nvecmin, self.nvecmax = nvecmin, nvecmax
        self.etrue = None

    def eigenvalues(self, on_block=None):
        v1 = initial_vector(self.run, self.emax)
        self.etrue, self.alpha, self.beta = lanczos_eigenvalues(self.hphi, v1, self.nkrymax, self.ntimes,
                                                                on_block)
        return self.etrue

    def eigenvectors(self):
        """cgradvecpar for the states nvecmin..min(nvecmax, ntrue), each from the
        initial guess (main_boundlanz.f:213-236).  Returns [(E, v, emean, its, ok)]."""
        if self.etrue is None:
            self.eigenvalues()
        v0 = initial_vector(self.run, self.emax)
        out = []
        for iv in range(self.nvecmin, min(self.nvecmax, len(self.etrue)) + 1):
            e = float(self.etrue[iv - 1])
            v, em, its, ok = cg_eigenvector(self.hphi, v0, e, self.nomxiter, self.criter)
            out.append((e, v, em, its, ok))
        return out
