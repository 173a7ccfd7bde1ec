"""Oracle and host set-up pinned against the reference's own golden log.

tests/golden/reference_pins.json is extracted from the reference's shipped
J=0 run (EXAMPLES/HD+H_collision/J000-check/sal.000) and README by
tests/golden/make_golden.py.  Every number here is independent of that run's
neural-network PES, so the restatements reproduce it from the namelist alone.
"""
import json
import math
import os

import pytest

from madwave3_gb300.host import constants as C
from madwave3_gb300.host import setup
from madwave3_gb300.host.wigner import gauleg
from oracle import mw3ref

PINS = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")))
NML = {k: float(v) if v.replace(".", "").replace("-", "").isdigit() else v for k, v in PINS["namelist"].items()}


def nml(k):
    return float(PINS["namelist"][k])


def masses():
    xm0, xm1, xm2 = nml("xm0"), nml("xm1"), nml("xm2")
    xmtot = xm0 + xm1 + xm2
    return xm0 * xm1 / (xm0 + xm1), xm2 * (xm0 + xm1) / xmtot


def ulps(a, b):
    return abs(a - b) / math.ulp(max(abs(a), abs(b)))


def test_gauss_legendre_140():
    w, x = gauleg(int(nml("nangu")))
    got = [math.acos(v) * 180.0 / C.pi for v in x]
    for g, r in zip(got, PINS["angles_deg_140"]):
        assert ulps(g, r) <= 2


def test_gauss_legendre_60_readme():
    w, x = gauleg(60)
    for i, r in PINS["angles_deg_60_head"]:
        assert ulps(math.acos(x[i - 1]) * 180.0 / C.pi, r) <= 2


def test_absorber_start():
    n = int(nml("npun1"))
    ah = (nml("rfin1") - nml("rmis1")) / (n - 1)
    _, ir1 = mw3ref.absorption(n, nml("rmis1"), ah, nml("absr1"), nml("absalp1"), int(nml("n1expo")), 1)
    _, ir2 = mw3ref.absorption(n, nml("rmis2"), ah, nml("absr2"), nml("absalp2"), int(nml("n2expo")), 1)
    assert [ir1, ir2] == PINS["ir1abs_ir2abs"]


def test_kinetic_energy_range():
    """Tradial's sinmom momenta: E_kin^2 for R (n = npun2) and E_kin^1 for r at the
    run's largest DST length (252 = 2^2 3^2 7, a noptFFT value)."""
    xm1red, xm2red = masses()
    n2 = int(nml("npun2"))
    ah2 = (nml("rfin2") - nml("rmis2")) / (n2 - 1)
    p2 = mw3ref.sinmom_p2((n2 - 1) * ah2, n2, xm2red, C.hbr) / C.conve1 / 8065.5
    assert ulps(p2.max(), PINS["ekin2max_ev"]) <= 1 and ulps(p2.min(), PINS["ekin2min_ev"]) <= 1
    n1 = 252
    assert mw3ref.noptfft(n1, int(nml("npun1"))) == n1
    ah1 = (nml("rfin1") - nml("rmis1")) / (int(nml("npun1")) - 1)
    p1 = mw3ref.sinmom_p2((n1 - 1) * ah1, n1, xm1red, C.hbr) / C.conve1 / 8065.5
    assert ulps(p1.max(), PINS["ekin1max_ev"]) <= 1 and ulps(p1.min(), PINS["ekin1min_ev"]) <= 1


def test_collision_packet():
    """set_colini: k0, alpha0 and the norm of the incident Gaussian on the R grid."""
    _, xm2red = masses()
    ecol = nml("ecol_ev") * C.eV2cm * C.conve1
    de = nml("deltae_ev") * C.eV2cm * C.conve1
    xk0 = math.sqrt(2.0 * xm2red * ecol) / C.hbr
    alpha0 = math.sqrt(2.0 * ecol / xm2red) * C.hbr / de
    assert xk0 == PINS["k0"] and alpha0 == PINS["alpha0"]
    factor0 = (2.0 / C.pi / alpha0 / alpha0) ** 0.25
    n2 = int(nml("npun2"))
    ah2 = (nml("rfin2") - nml("rmis2")) / (n2 - 1)
    s = sum(setup.rgauscolini(nml("rmis2") + i * ah2, nml("rcolini_ang"), alpha0, xk0, factor0) ** 2
            for i in range(n2)) * ah2
    assert abs(s - PINS["gauss_norm"]) <= 4e-16


def test_smatini_energy_norm():
    """Smatini_col: energy distribution of the packet (Riccati-Bessel projection)."""
    _, xm2red = masses()
    ecol = nml("ecol_ev") * C.eV2cm * C.conve1
    de = nml("deltae_ev") * C.eV2cm * C.conve1
    xk0 = math.sqrt(2.0 * xm2red * ecol) / C.hbr
    alpha0 = math.sqrt(2.0 * ecol / xm2red) * C.hbr / de
    factor0 = (2.0 / C.pi / alpha0 / alpha0) ** 0.25
    xm1reac = masses()[0]
    xn, et, ap, rf = mw3ref.smatini_col(int(nml("netot")), nml("ekinmin_ev") * C.eV2cm * C.conve1,
                                        nml("ekinmax_ev") * C.eV2cm * C.conve1, nml("rmis2"), nml("rfin2"),
                                        nml("rcolini_ang"), xk0, alpha0, factor0, xm2red, xm1reac, 0, C.hbr)
    assert abs(xn - PINS["norm_in_energy"]) / PINS["norm_in_energy"] < 1e-12


def test_energy_interval():
    """pot2: Emax = Vmax + radcut + 3 rotcut with Vmax = Vcut for one state."""
    emax = nml("vcutmaxev") + nml("radcutmaxev") + 3 * nml("rotcutmaxev")
    z = (nml("vcutmaxev") * C.eV2cm * C.conve1 + nml("radcutmaxev") * C.eV2cm * C.conve1
         + 3.0 * nml("rotcutmaxev") * C.eV2cm * C.conve1)
    assert z / C.conve1 / C.eV2cm == pytest.approx(PINS["emax_ev"], rel=1e-15) == emax


def test_flux_line_index(tmp_path):
    """ini_flux: ir4flux on the log's r1 grid (only the radial grid matters)."""
    from madwave3_gb300.host import generator
    d = str(tmp_path / "fluxgrid")
    generator.write_case(d, npun1=int(nml("npun1")), rmis1=nml("rmis1"), rfin1=nml("rfin1"), npun1min=8,
                         npun2=48, nangu=4, jmax=3, nvmax=1, netot=8, r1flux_bohr=nml("r1flux_ang") / C.convl)
    run = setup.load(os.path.join(d, "input.dat"))
    assert mw3ref.Oracle(run).flux_tables()["ir4flux"] == PINS["ir4flux"]
