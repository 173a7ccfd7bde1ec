"""Synthetic input generator: the ``pot.out`` equivalent for LEPS surfaces.

Writes ``pot/cont.pot``, ``pot/pot.NNN.dat``, ``func/bcwf``, ``func/eref``
and ``input.dat`` in the formats the reference reads
(pot/cont.pot: SRC/mod_pot_01y2.f:292-303; pot/pot.NNN.dat rows
``ir1 ir2 ((V(ie,je),ie),je)``: :275-276, read :472-494; func/bcwf:
SRC/mod_baseYfunciones_01y2.f:797-808; func/eref: :788-790).

The potential is a London-Eyring-Polanyi-Sato surface built from one Morse
pair potential shared by the three atom pairs (D, beta, r_e in eV and
angstrom, Sato parameter k)::

    1E(r) = D (exp(-2b(r-re)) - 2 exp(-b(r-re)))        singlet
    3E(r) = D/2 (exp(-2b(r-re)) + 2 exp(-b(r-re)))      anti-bonding triplet
    Q_i   = (1E_i (1+k) + 3E_i (1-k)) / 2,  J_i = (1E_i (1+k) - 3E_i (1-k)) / 2
    V     = (Q_1+Q_2+Q_3 - sqrt(((J1-J2)^2 + (J2-J3)^2 + (J3-J1)^2) / 2)) / (1+k)

which tends to the singlet Morse curve of a pair when the third atom leaves.
Compression follows pot1 (SRC/mod_pot_01y2.f:147-341): a grid point is kept
when at least one adiabatic energy lies below Vcut, diagonal entries above
Vcut are capped with their row/column zeroed, and V is referred to the
energy of the reactant (v=0, j=0) diatomic level.

Diatomic functions fd(r1; v, j) are eigenvectors of a sine-DVR Hamiltonian
on exactly the r1 grid of the propagation (the same sine basis the radial
kinetic operator uses), normalised to sum(fd^2) = 1 as the reference's
files are.  The reference obtains them by Numerov shooting instead; both
sides of the parity tests read these same files, so that difference does not
enter any comparison.
"""
import math
import os

import numpy as np

from . import constants as C
from . import namelist

BOHR = C.convl  # angstrom per bohr
SADDLE_R = 0.93  # angstrom: symmetric collinear saddle of the LEPS surface below


def morse_singlet(r, D, beta, re):
    x = np.exp(-beta * (r - re))
    return D * (x * x - 2.0 * x)


def morse_triplet(r, D, beta, re):
    x = np.exp(-beta * (r - re))
    return 0.5 * D * (x * x + 2.0 * x)


def leps(r01, r02, r12, D=4.75, beta=1.94, re=0.74, k=0.17):
    """LEPS energy in eV for the three interatomic distances in angstrom."""
    Q, J = [], []
    for r in (r01, r02, r12):
        s = morse_singlet(r, D, beta, re)
        t = morse_triplet(r, D, beta, re)
        Q.append(0.5 * (s * (1 + k) + t * (1 - k)))
        J.append(0.5 * (s * (1 + k) - t * (1 - k)))
    exch = np.sqrt(0.5 * ((J[0] - J[1]) ** 2 + (J[1] - J[2]) ** 2 + (J[2] - J[0]) ** 2))
    return (Q[0] + Q[1] + Q[2] - exch) / (1 + k)


def jacobi_distances(r, R, cg, xm0, xm1):
    """Atom-pair distances for reactant Jacobi (r = 0-1, R = 2 to CM(01), cos gamma)."""
    gam = xm1 / (xm0 + xm1)
    r02 = np.sqrt(R * R + gam * gam * r * r + 2.0 * gam * R * r * cg)
    g1 = 1.0 - gam
    r12 = np.sqrt(np.maximum(R * R + g1 * g1 * r * r - 2.0 * g1 * R * r * cg, 0.0))
    return r, r02, r12


def sine_dvr_states(rgrid, V, mu, nstates):
    """Lowest eigenpairs of -hbar^2/2mu d2/dr2 + V on the given uniform grid."""
    n = len(rgrid)
    ah = rgrid[1] - rgrid[0]
    L = (n + 1) * ah
    kk = np.arange(1, n + 1) * math.pi / L
    S = math.sqrt(2.0 / (n + 1)) * np.sin(np.outer(np.arange(1, n + 1), np.arange(1, n + 1)) * math.pi / (n + 1))
    T = (S * (C.hbr ** 2 * kk ** 2 / (2.0 * mu))) @ S
    H = T + np.diag(V)
    e, v = np.linalg.eigh(H)
    v = v[:, :nstates]
    for c in range(v.shape[1]):             # sign: positive at the largest lobe
        if v[np.argmax(np.abs(v[:, c])), c] < 0:
            v[:, c] = -v[:, c]
    return e[:nstates], v


DEFAULT = dict(
    # grid: R in [0.1,15] bohr, r in [0.5,12] bohr, as the workloads state
    npun1=128, rmis1=0.5 * BOHR, rfin1=12.0 * BOHR, npun1min=32,
    npun2=256, rmis2=0.1 * BOHR, rfin2=15.0 * BOHR,
    nangu=60, Jtot=0, iparity=1, inc=1, nelecmax=1, iommin=0, iommax=0, j0=0,
    jini=0, jmax=20, nvini=0, nvmax=5, nvref=0, jref=0, iomref=0, ielecref=1,
    xm0=2.014, xm1=1.008, xm2=1.008,
    vcutmaxev=2.5, radcutmaxev=2.5, rotcutmaxev=5.0,
    n1expo=3, n2expo=3, ninterv1=1, ninterv2=1,
    rcolini_bohr=9.0, ecol_ev=0.5, alpha0_bohr=0.3,
    netot=1000, ekinmin_ev=0.1, ekinmax_ev=1.5, r1flux_bohr=8.5,
    ntimes=500, nloop=3, kminelastic=0,
    shifts_ev=(0.0, 0.8, 1.5), coupling_ev=0.05, coupling_width_bohr=0.5,
    absorb_strength=10.0,
    iphoto=0,
    lambdas=None,        # Omega_diatom (Lambda) of each electronic state; None: all 0
)


def make_inputs(**over):
    """Namelist groups for one case; absorber over the outer 20 % of R and r,
    cubic, with absalp chosen so the damping exponent reaches
    ``absorb_strength`` at the grid edge."""
    p = dict(DEFAULT)
    p.update(over)
    absr1 = p["rmis1"] + 0.8 * (p["rfin1"] - p["rmis1"])
    absr2 = p["rmis2"] + 0.8 * (p["rfin2"] - p["rmis2"])
    absalp1 = p["absorb_strength"] / (p["rfin1"] - absr1) ** p["n1expo"]
    absalp2 = p["absorb_strength"] / (p["rfin2"] - absr2) ** p["n2expo"]
    xm0, xm1, xm2 = p["xm0"], p["xm1"], p["xm2"]
    xm2reac = xm2 * (xm0 + xm1) / (xm0 + xm1 + xm2)
    ecol = p["ecol_ev"] * C.eV2cm * C.conve1
    alpha0 = p["alpha0_bohr"] * BOHR
    deltae = math.sqrt(2.0 * ecol / xm2reac) * C.hbr / alpha0       # mod_colini_01y2.f:56-58
    deltae_ev = deltae / C.conve1 / C.eV2cm
    g = {
        "inputgridbase": dict(
            npun1=p["npun1"], rmis1=p["rmis1"], rfin1=p["rfin1"], npun1min=p["npun1min"],
            npun2=p["npun2"], rmis2=p["rmis2"], rfin2=p["rfin2"], nangu=p["nangu"],
            jtot=p["Jtot"], iparity=p["iparity"], inc=p["inc"], nelecmax=p["nelecmax"],
            iommin=p["iommin"], iommax=p["iommax"], j0=p["j0"], jini=p["jini"], jmax=p["jmax"],
            nvini=p["nvini"], nvmax=p["nvmax"], nvref=p["nvref"], jref=p["jref"],
            iomref=p["iomref"], ielecref=p["ielecref"]),
        "inputprod": dict(iprod=0),
        "inputprocess": dict(iphoto=p["iphoto"]),
        "inputpotmass": dict(system="H+DH LEPS", xm0=xm0, xm1=xm1, xm2=xm2,
                             vcutmaxev=p["vcutmaxev"], radcutmaxev=p["radcutmaxev"],
                             rotcutmaxev=p["rotcutmaxev"]),
        "inputabsorcion": dict(absr1=absr1, absalp1=absalp1, n1expo=p["n1expo"], ninterv1=p["ninterv1"],
                               absr2=absr2, absalp2=absalp2, n2expo=p["n2expo"], ninterv2=p["ninterv2"]),
        "inputcol": dict(rcolini_ang=p["rcolini_bohr"] * BOHR, ecol_ev=p["ecol_ev"], deltae_ev=deltae_ev),
        "inputflux": dict(r1flux_ang=p["r1flux_bohr"] * BOHR, netot=p["netot"],
                          ekinmin_ev=p["ekinmin_ev"], ekinmax_ev=p["ekinmax_ev"], ncontfile=0),
        "inputtime": dict(ntimes=p["ntimes"], nloop=p["nloop"], kminelastic=p["kminelastic"]),
    }
    return g, p


def diabatic_matrix(r01, r02, r12, p):
    """nelec x nelec diabatic matrix (eV) on arrays of geometries."""
    ne = p["nelecmax"]
    base = leps(r01, r02, r12)
    V = np.zeros((ne, ne) + np.shape(base))
    for e in range(ne):
        V[e, e] = base + p["shifts_ev"][e]
    if ne > 1:
        # Gaussian couplings centred on the product-channel saddle region
        # (r02 short, r01 stretched), non-zero only in the 02+1 channel.
        rs = SADDLE_R
        w = p["coupling_width_bohr"] * BOHR
        gauss = p["coupling_ev"] * np.exp(-((r02 - rs) ** 2 + (r01 - rs) ** 2) / (w * w))
        gauss = np.where(r01 > r02, gauss, 0.0)
        for a in range(ne):
            for b in range(a + 1, ne):
                V[a, b] = gauss
                V[b, a] = gauss
    return V


def write_case(outdir, **over):
    """Generate input.dat, pot/ and func/ for one case; returns the parameters."""
    groups, p = make_inputs(**over)
    os.makedirs(os.path.join(outdir, "pot"), exist_ok=True)
    os.makedirs(os.path.join(outdir, "func"), exist_ok=True)
    with open(os.path.join(outdir, "input.dat"), "w") as f:
        f.write(namelist.dumps(groups))
    write_func(outdir, p)
    write_pot(outdir, p)
    return p


def write_func(outdir, p):
    ne = p["nelecmax"]
    n1 = p["npun1"]
    ah1 = (p["rfin1"] - p["rmis1"]) / (n1 - 1)
    r = p["rmis1"] + ah1 * np.arange(n1)
    xm1red = p["xm0"] * p["xm1"] / (p["xm0"] + p["xm1"])
    far = 100.0
    nv = p["nvmax"] + 1
    lines = []
    eref = None
    for ie in range(ne):
        Vd = diabatic_matrix(r, np.full_like(r, far), np.full_like(r, far), p)[ie, ie]
        Vd = Vd * C.eV2cm * C.conve1
        for j in range(p["jini"], p["jmax"] + 1):
            cent = j * (j + 1) * C.hbr ** 2 / (2.0 * xm1red * r * r)
            e, v = sine_dvr_states(r, Vd + cent, xm1red, nv)
            if ie == p["ielecref"] - 1 and j == p["jref"]:
                eref = e[p["nvref"]]
            lines.append("%d %d %d" % (ie + 1, j, p["nvmax"]))
            for iv in range(p["nvini"], p["nvmax"] + 1):
                lines.append("%d %s" % (iv, repr(float(e[iv]))))
                lines.extend(repr(float(x)) for x in v[:, iv])
    with open(os.path.join(outdir, "func", "bcwf"), "w") as f:
        f.write("\n".join(lines) + "\n")
    with open(os.path.join(outdir, "func", "eref"), "w") as f:
        f.write(repr(float(eref)) + "\n")
    p["_eref"] = eref


def product_states(run, n2prod1, jiniprod, jmaxprod, nviniprod, nvmaxprod, **over):
    """The product diatom's (atoms 0-2, atom 1 far away) states on the R grid,
    as product_radialf_read builds them for diabatic products
    (SRC/mod_baseYfunciones_01y2.f:1085-1250): the coupled nelec-state sine DVR
    of the 02 diatom per j, each state discrete-normalised over the grid and
    kept on its first n2prod1 points.  ``over`` are the case's generator
    parameters (for the surface).  Returns (fdprod[njp][nvp][nelec][n2prod1],
    ediatprod[njp][nvp] in zot, nobcprod[njp] = noBCprod(jiniprod:jmaxprod),
    nviniprod - 1 where no state is bound)."""
    _, p = make_inputs(**over)
    inp = run.inp
    n = inp.npun2
    ah = run.ah2
    r = inp.rmis2 + ah * np.arange(n)
    far = np.full_like(r, 100.0)
    ne = run.nelec
    V = diabatic_matrix(far, r, far, p) * C.eV2cm * C.conve1          # [ne][ne][n], zot
    mu = run.xm1prod
    L = (n + 1) * ah
    kk = np.arange(1, n + 1) * math.pi / L
    S = math.sqrt(2.0 / (n + 1)) * np.sin(np.outer(np.arange(1, n + 1), np.arange(1, n + 1)) * math.pi / (n + 1))
    T = (S * (C.hbr ** 2 * kk ** 2 / (2.0 * mu))) @ S
    asym = min(V[e, e, -1] for e in range(ne))
    njp, nvp = jmaxprod - jiniprod + 1, nvmaxprod - nviniprod + 1
    fd = np.zeros((njp, nvp, ne, n2prod1))
    ed = np.zeros((njp, nvp))
    nob = np.full(njp, nviniprod - 1, np.int32)
    for jj, j in enumerate(range(jiniprod, jmaxprod + 1)):
        cent = j * (j + 1) * C.hbr ** 2 / (2.0 * mu * r * r)
        H = np.zeros((ne * n, ne * n))
        for e in range(ne):
            H[e * n:(e + 1) * n, e * n:(e + 1) * n] = T + np.diag(cent)
            for f in range(ne):
                H[e * n:(e + 1) * n, f * n:(f + 1) * n] += np.diag(V[e, f])
        w, v = np.linalg.eigh(H)
        nbound = int(np.sum(w < asym))
        nob[jj] = min(nbound - 1, nvmaxprod) if nbound - 1 >= nviniprod else nviniprod - 1
        for vv, iv in enumerate(range(nviniprod, nvmaxprod + 1)):
            c = v[:, iv]
            if c[np.argmax(np.abs(c))] < 0:
                c = -c
            ed[jj, vv] = w[iv]
            fd[jj, vv] = c.reshape(ne, n)[:, :n2prod1]
    return fd, ed, nob


def write_pot(outdir, p):
    from .wigner import gauleg
    n1, n2, na, ne = p["npun1"], p["npun2"], p["nangu"], p["nelecmax"]
    ah1 = (p["rfin1"] - p["rmis1"]) / (n1 - 1)
    ah2 = (p["rfin2"] - p["rmis2"]) / (n2 - 1)
    r1 = p["rmis1"] + ah1 * np.arange(n1)
    r2 = p["rmis2"] + ah2 * np.arange(n2)
    w, x = gauleg(na * p["inc"])
    vcut = p["vcutmaxev"] * C.eV2cm * C.conve1
    vref = p["_eref"]
    vmin = 1e10
    vmaxtot = vcut
    npunreal = []
    maxpoint = 0
    RR, rr = np.meshgrid(r2, r1, indexing="ij")           # [ir2, ir1]: ir1 fastest as pot1 loops
    for iang in range(na):
        a, b, c = jacobi_distances(rr, RR, x[iang], p["xm0"], p["xm1"])
        V = diabatic_matrix(a, b, c, p) * C.eV2cm * C.conve1   # [ne,ne,n2,n1]
        for e in range(ne):
            V[e, e] -= vref
        # cap diagonal entries above Vcut (row/column zeroed)
        for e in range(ne):
            hi = V[e, e] > vcut
            for f in range(ne):
                V[e, f] = np.where(hi, 0.0, V[e, f])
                V[f, e] = np.where(hi, 0.0, V[f, e])
            V[e, e] = np.where(hi, vcut, V[e, e])
        if ne == 1:
            eig = V[0, 0][None]
        else:
            Vm = np.moveaxis(V, (0, 1), (-2, -1))
            eig = np.moveaxis(np.linalg.eigvalsh(Vm), -1, 0)
        vmaxtot = max(vmaxtot, float(eig.max()))
        vmin = min(vmin, float(eig.min()))
        keep = (eig < vcut).any(axis=0)                   # [n2, n1]
        i2, i1 = np.nonzero(keep)                        # row-major: ir2 outer, ir1 inner
        rows = [np.stack([i1 + 1, i2 + 1], 1).astype(float)]
        for je in range(ne):
            for ie in range(ne):
                rows.append(V[ie, je][i2, i1][:, None])
        data = np.hstack(rows)
        with open(os.path.join(outdir, "pot", "pot.%03d.dat" % (iang + 1)), "w") as f:
            for row in data:
                f.write("%d %d %s\n" % (int(row[0]), int(row[1]),
                                       " ".join(repr(float(v)) for v in row[2:])))
        npunreal.append(len(i1))
        maxpoint += len(i1)
    with open(os.path.join(outdir, "pot", "cont.pot"), "w") as f:
        f.write("%d\n" % ne)
        lam = p.get("lambdas") or (0,) * ne
        for e in range(ne):
            f.write("%d 0 1.0 1.0\n" % lam[e])
        f.write("%r %d %r\n" % (vmin, maxpoint, vmaxtot))
        f.write("%r %r %d\n" % (p["rmis1"], p["rfin1"], n1))
        f.write("%r %r %d\n" % (p["rmis2"], p["rfin2"], n2))
        f.write("%d %d\n" % (na, p["inc"]))
        f.write(" ".join("%d" % n for n in npunreal) + "\n")


# Named workloads (grid sizes, blocks, iterations) ---------------------------
CASES = {
    # J=0, one Omega block, one state: 256 R x 128 r x 60 angles, 2000 iterations
    "j0_256x128x60": dict(),
    # larger J=0 grid: 512 R x 256 r x 120 angles, 10000 iterations
    "j0_512x256x120": dict(npun2=512, npun1=256, nangu=120, jmax=39),
    # J=10, Omega = 0..10 Coriolis-coupled: 11 blocks x 256 x 128 x 60
    "j10_256x128x60": dict(Jtot=10, iommax=10),
    # three diabatic states, Omega=0..2 (J=2): 384 R x 192 r x 80 angles
    "e3_384x192x80": dict(npun2=384, npun1=192, nangu=80, nelecmax=3, Jtot=2, iommax=2),
    # small cases the parity tests run on the CPU oracle
    "tiny_j0": dict(npun2=40, npun1=24, nangu=10, jmax=6, nvmax=2, netot=64, npun1min=8,
                    alpha0_bohr=1.2),
    "tiny_j3": dict(npun2=40, npun1=24, nangu=10, jmax=6, nvmax=2, netot=64, npun1min=8,
                    Jtot=3, iommax=3, iparity=-1, alpha0_bohr=1.2),
    "tiny_e2": dict(npun2=36, npun1=20, nangu=8, jmax=5, nvmax=2, netot=48, npun1min=8,
                    nelecmax=2, Jtot=1, iommax=1, iparity=-1, alpha0_bohr=1.2, shifts_ev=(0.0, 0.3), coupling_ev=0.2,
                    coupling_width_bohr=1.5),
    # two coupled states with Lambda = 0 and 1 (same sigma), J = 2, Omega = 0..2: the
    # channels of equal Omega couple through the electronic Coriolis term
    "tiny_ecor": dict(npun2=36, npun1=20, nangu=8, jmax=5, nvmax=2, netot=48, npun1min=8,
                      nelecmax=2, lambdas=(0, 1), Jtot=2, iommax=2, iparity=1, alpha0_bohr=1.2,
                      shifts_ev=(0.0, 0.3), coupling_ev=0.2, coupling_width_bohr=1.5),
    # three states with Lambda = 0, 1, 0: each Lambda = 1 channel couples to two sources
    "tiny_ecor3": dict(npun2=32, npun1=20, nangu=8, jmax=5, nvmax=2, netot=48, npun1min=8,
                       nelecmax=3, lambdas=(0, 1, 0), Jtot=2, iommax=2, iparity=1, alpha0_bohr=1.2,
                       shifts_ev=(0.0, 0.3, 0.5), coupling_ev=0.2, coupling_width_bohr=1.5),
}


def jsweep_inputs(J, **over):
    """Per-J settings of the partial-wave sweep J=0..40 with Omega_max=min(J,6).

    The total parity is set to (-1)^J, the parity of the H + HD(v=0, j=0)
    entrance channel with l = J, so the Omega=0 block (which the basis drops
    when iparity differs from sigma (-1)^J, mod_baseYfunciones_01y2.f:143-145)
    is present for every J and the sweep has sum_J (min(J,6)+1) = 266 blocks."""
    return dict(Jtot=J, iparity=(-1) ** J, iommin=0, iommax=min(J, 6), iomref=0, **over)
