"""Photodissociation spectra from the Chebyshev autocorrelation, as the
post-processing program cheby-spectra does (SRC/photo/cheby-spectra.f).

The propagation of a photodissociation wave writes auto.vVV.jJJ.JJJJ (header:
photonorm, the initial bound state's energy in eV, emindlt and delta2 in
zots; then one 'k <psi0|psi_k>' line per iteration; madwave3_gb300.photo).
The program reads it with auto(0) = 1 and, on an equispaced grid of ne
energies E in [Emin, Emax] (eV, relative to the reference energy eref of
func/eref), forms the damped modified Chebyshev transform

    s(E) = hbar [auto(0) + 2 sum_k cos(k acos Es) exp(-k xkgam) auto(k)]
           / (sqrt(1 - Es^2) delta2),         Es = (E - emindlt) / delta2,

(0 where it is not a number, i.e. |Es| > 1), and from it
    spectrum_au = s photonorm / (pi hbar zot2au)          (1 / hartree),
    photon energy = (E + eref - E_bound) / au2eV           (hartree),
    cross section = photon energy x spectrum_au / (c epsilon0)   (atomic units),
and the integral sum(spectrum_au / photonorm) dE, which is 1 for a spectrum
the grid resolves (:55-99).  Units and constants are the program's own.
"""
import math

import numpy as np

# cheby-spectra.f:36-49
CONVE1 = 1.197e-4
CONVL = 0.52917726
CONVE = 4.55633538e-6
CONVM = 0.182288853e4
EV2CM = 8065.5
AU2EV = 27.21113957
ZOT2AU = (1.0 / CONVE1) * CONVE
HBR = CONVL / math.sqrt(CONVM * CONVE / CONVE1)
CLUZ_AU = 137.0
EPSILON0_AU = 0.07957747
CS_CONSTANT_AU = 1.0 / (CLUZ_AU * EPSILON0_AU)


def _float(tok):
    return float(tok.replace("D", "E").replace("d", "e"))


def read_auto_file(path, kmax=None):
    """(photonorm, E_bound in eV, emindlt, delta2, auto[0..kmaxreal]) of an
    auto file, read as the program does (:59-65): auto(0) = 1 and auto(k) at the
    k each line names, at most kmax lines."""
    with open(path) as f:
        head = f.readline().split()
        xnorm, ebndini, emindlt, delta2 = (_float(t) for t in head[:4])
        ks, vals = [], []
        for line in f:
            t = line.split()
            if len(t) < 2:
                continue
            if kmax is not None and len(ks) >= kmax:
                break
            ks.append(int(t[0]))
            vals.append(_float(t[1]))
    kmaxreal = ks[-1] if ks else 0
    auto = np.zeros(max(kmaxreal, max(ks, default=0)) + 1)
    auto[0] = 1.0
    auto[np.array(ks, dtype=np.int64)] = vals
    return xnorm, ebndini, emindlt, delta2, auto[:kmaxreal + 1]


def spectrum(auto, xnorm, ebndini, emindlt, delta2, eref_zot, emin_ev, emax_ev, ne, xkgam):
    """The program's table (:67-99) as arrays: E (eV), s photonorm, the cross
    section (a.u.), the photon energy (hartree), spectrum_au, and the integral."""
    auto = np.asarray(auto, dtype=np.float64)
    kmaxreal = len(auto) - 1
    eshift = eref_zot / (CONVE1 * EV2CM)
    estep = (emax_ev - emin_ev) / float(ne - 1)
    ee = emin_ev + np.arange(ne, dtype=np.float64) * estep
    es = (ee * EV2CM * CONVE1 - emindlt) / delta2
    k = np.arange(1, kmaxreal + 1, dtype=np.float64)
    w = 2.0 * HBR * np.exp(-k * xkgam) * auto[1:]
    s = np.empty(ne)
    chunk = max(1, 4_000_000 // max(kmaxreal, 1))      # energies per block of cos(k theta) terms
    # |Es| > 1 gives NaN, set to 0 as the program does; |Es| = 1 exactly divides by zero
    # and stays infinite there, as in the program (isnan does not catch it)
    with np.errstate(invalid="ignore", divide="ignore"):
        theta = np.arccos(es)
        deno = np.sqrt(1.0 - es * es)
        for i0 in range(0, ne, chunk):
            th = theta[i0:i0 + chunk]
            s[i0:i0 + chunk] = auto[0] * HBR + np.cos(np.outer(th, -k)) @ w
        s = s / (deno * delta2)
    s = np.where(np.isnan(s), 0.0, s)
    ephoton = (ee + eshift - ebndini) / AU2EV
    spec_au = s * xnorm / (math.pi * HBR * ZOT2AU)
    integral = float(np.sum(spec_au / xnorm)) * estep / AU2EV
    return {"E_ev": ee, "spectrum": s * xnorm, "xsection_au": CS_CONSTANT_AU * ephoton * spec_au,
            "ephoton_au": ephoton, "spectrum_au": spec_au, "integral": integral}


def write_table(path, sp):
    """The program's output lines (20(1x,e15.7)) and its closing integral line."""
    with open(path, "w") as f:
        for row in zip(sp["E_ev"], sp["spectrum"], sp["xsection_au"], sp["ephoton_au"], sp["spectrum_au"]):
            f.write("".join(" %15.7E" % v for v in row + (CS_CONSTANT_AU,)) + "\n")
        f.write("  integral= %r\n" % sp["integral"])


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser(description="absorption spectrum from an auto file (cheby-spectra)")
    ap.add_argument("auto")
    ap.add_argument("--eref-file", default="../func/eref", help="func/eref of the case (zots)")
    ap.add_argument("--emin", type=float, required=True, help="eV")
    ap.add_argument("--emax", type=float, required=True, help="eV")
    ap.add_argument("--ne", type=int, required=True)
    ap.add_argument("--xkgam", type=float, required=True)
    ap.add_argument("--kmax", type=int, default=None)
    ap.add_argument("--out", default="-")
    a = ap.parse_args(argv)
    with open(a.eref_file) as f:
        eref = _float(f.read().split()[0])
    xnorm, eb, emin_d, d2, auto = read_auto_file(a.auto, a.kmax)
    sp = spectrum(auto, xnorm, eb, emin_d, d2, eref, a.emin, a.emax, a.ne, a.xkgam)
    if a.out == "-":
        import sys
        for row in zip(sp["E_ev"], sp["spectrum"], sp["xsection_au"], sp["ephoton_au"], sp["spectrum_au"]):
            sys.stdout.write("".join(" %15.7E" % v for v in row + (CS_CONSTANT_AU,)) + "\n")
        sys.stdout.write("  integral= %r\n" % sp["integral"])
    else:
        write_table(a.out, sp)


if __name__ == "__main__":
    main()
