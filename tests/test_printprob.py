"""printprob's files (SRC/main_madwave3.f:555-844): Fortran E formats, the
S2prod / S2prodelec layout for iprod = 0 from the oracle's accumulators, and
the reader against the layout of the reference's shipped S2prod file."""
import json
import os

import numpy as np

from madwave3_gb300 import printprob
from madwave3_gb300.host.constants import conve1, eV2cm, pi

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "reference_pins.json")


def test_fortran_e_formats():
    assert printprob.e17_7e3(0.1) == "   0.1000000E+000"
    assert printprob.e17_7e3(-0.0123456789) == "  -0.1234568E-001"
    assert printprob.e17_7e3(0.99999999) == "   0.1000000E+001"
    assert printprob.e17_7e3(1.0e-95) == "   0.1000000E-094"
    assert printprob.e17_7e3(0.0) == "   0.0000000E+000"
    assert printprob.fortran_e(0.0028056112, 15, 7) == "  0.2805611E-02"


def test_reader_takes_the_reference_layout():
    """The shipped S2prod (e15.7 columns, iprod = 2: E, P, P + S2reac, S2no and
    the v' distribution) parses to its 15 columns; its energy column is the
    grid ekinmin + (ie - 1) (ekinmax - ekinmin) / (netot - 1) that etot follows."""
    g = json.load(open(GOLDEN))
    s = g["s2prod"]
    a = np.array([[float(x) for x in l.split()] for l in s["head"] + s["tail"]])
    assert a.shape == (4, s["columns"]) and s["columns"] == 15 and s["lines"] == 500
    nml = g["namelist"]
    emin, emax, n = float(nml["ekinmin_ev"]), float(nml["ekinmax_ev"]), int(nml["netot"])
    e = emin + np.array([0, 1, 2, n - 1]) * (emax - emin) / (n - 1)
    assert np.allclose(a[:, 0], e, rtol=5.01e-7, atol=0)
    # the same energies through this writer's format read back to the same values
    ours = np.array([float(printprob.e17_7e3(x)) for x in e])
    assert np.array_equal(ours, a[:, 0])


def test_s2prod_from_oracle(runs, tmp_path):
    from oracle.mw3ref import Oracle

    run = runs["tiny_j3"]
    i = run.inp
    o = Oracle(run)
    o.start(run.psi0)
    o.run_iters(60)
    tot, el = o.totalflux()
    zs2, _ = o.s2()
    ft = o.flux_tables()
    s2f = o.s2factor()
    path = printprob.write_s2prod(str(tmp_path), run, 1, tot, el, zs2, ft["etot"], ft["reacfct"], s2f)
    assert os.path.basename(path) == "S2prod.v%02d.J%03d.k00001" % (i.nvref, i.Jtot)
    lines = open(path).read().splitlines()
    assert len(lines) == i.netot and all(len(l) == 4 * 18 for l in lines)
    a = printprob.read_s2prod(path)
    # S2reac summed directly over the (block, j, v) elements printprob takes
    mask = np.zeros(zs2.shape[:3], bool)
    for b in range(run.ncan):
        e = run.nelebas[b] - 1
        for j in range(run.j00[b], i.jmax + 1, i.inc):
            mask[b, j - i.jini, : run.nobc[e, j - i.jini] - i.nvini + 1] = True
    fac = s2f[np.asarray(run.nelebas) - 1]                      # [ncan][nj][nv][netot]
    s2reac = (np.abs(zs2 / (2 * pi)) ** 2 * fac * mask[..., None]).sum(axis=(0, 1, 2))
    assert np.any(s2reac > 1e-12)
    np.testing.assert_allclose(a[:, 0], ft["etot"] / conve1 / eV2cm, rtol=5.01e-7)
    np.testing.assert_allclose(a[:, 1], np.where(tot < 1e-90, 0, tot), rtol=5.01e-7, atol=1e-300)
    np.testing.assert_allclose(a[:, 2], np.where(tot < 1e-90, 0, tot) + np.where(s2reac < 1e-90, 0, s2reac),
                               rtol=5.01e-7, atol=1e-300)
    np.testing.assert_allclose(a[:, 3], ft["reacfct"], rtol=5.01e-7, atol=1e-300)
    b = printprob.read_s2prod(os.path.join(str(tmp_path), "S2prodelec"))
    assert b.shape == (i.netot, 1 + run.nelec)
    np.testing.assert_allclose(b[:, 1:], el.T, rtol=5.01e-7, atol=1e-300)


def test_s2prod_iprod2_layout_matches_the_shipped_file(runs, tmp_path):
    """iprod = 2 from the oracle's product projection (seeded tables with
    v' = 0..10, as in the shipped run): 15 columns like the reference's
    S2prod.v00.J000.k00008; S2no and the v' columns are the S2pro sums."""
    from dataclasses import replace

    from conftest import synthetic_product_tables
    from oracle.mw3ref import Oracle

    g = json.load(open(GOLDEN))["s2prod"]
    run = runs["tiny_j3"]
    i = run.inp
    pp = synthetic_product_tables(run)
    rng = np.random.default_rng(7)
    njp = pp.jmaxprod - pp.jiniprod + 1
    pp = replace(pp, nvmaxprod=10, nobcprod=rng.integers(0, 11, njp).astype(np.int32),
                 prodwf=rng.standard_normal(pp.prodwf.shape[:2] + (11,) + pp.prodwf.shape[3:]))
    o = Oracle(run)
    o.set_product(pp)
    o.start(run.psi0)
    o.run_iters(20)
    zp, _ = o.product()
    fac = rng.uniform(0.5, 2.0, (njp, 11, i.netot))
    tot, el = o.totalflux()
    zs2, _ = o.s2()
    ft = o.flux_tables()
    path = printprob.write_s2prod(str(tmp_path), run, 3, tot, el, zs2, ft["etot"], ft["reacfct"], o.s2factor(),
                                  iprod=2, product=(zp, fac, pp))
    a = printprob.read_s2prod(path)
    assert a.shape == (i.netot, g["columns"])
    s2pro = np.abs(zp) ** 2 / (4 * pi * pi) * fac[None]
    for jj in range(njp):
        s2pro[:, jj, pp.nobcprod[jj] + 1:] = 0
    vib = s2pro.sum(axis=(0, 1))
    vib = np.where(vib < 1e-90, 0, vib)
    np.testing.assert_allclose(a[:, 4:], vib.T, rtol=5.01e-7, atol=1e-300)
    np.testing.assert_allclose(a[:, 3], vib.sum(axis=0), rtol=5.01e-7, atol=1e-300)
    assert np.any(a[:, 3] > 0)
