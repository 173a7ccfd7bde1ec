"""distriwvp (SRC/AUXILIARy-CODES/distriwvp.f, iprod = 2) restated: the
per-iteration Cvjprod records the propagation writes, read back and
transformed to energy, against the oracle's own accumulators; its packet
distribution against the oracle's Smatini_col; the distribution tables
against a direct transcription of the program's loops; the whole program on a
generated case directory."""
import math
import os

import numpy as np
import pytest

from conftest import synthetic_product_tables
from madwave3_gb300 import contfiles, distri
from madwave3_gb300.host import constants as C
from madwave3_gb300.host import namelist, potini
from oracle.mw3ref import Oracle

NIT = 40


def oracle_history(run, n=NIT):
    """The oracle with the seeded product projection: Cvjprod of each of the n
    iterations, and zS2prod after them."""
    pp = synthetic_product_tables(run)
    o = Oracle(run)
    o.set_product(pp)
    o.start(run.psi0)
    rows = []
    for _ in range(n):
        o.run_iters(1)
        rows.append(o.product()[1].copy())
    return pp, o, np.array(rows)


def test_records_rebuild_the_accumulators(runs, tmp_path):
    run = runs["tiny_j3"]
    pp, o, rows = oracle_history(run)
    # the propagation's iterations after a fresh start are 2, 3, ... (its records' numbers)
    contfiles.write_cvj_file(str(tmp_path / "Cvjprod.0001"), range(2, NIT + 2), rows)
    rec = distri.read_records(str(tmp_path), 1, NIT, rows.shape[1:])
    assert np.array_equal(rec, rows)
    etot = o.flux_tables()["etot"]
    z = distri.chebyshev_sum(rec, etot, run.emindlt, run.delta2, hbr=C.hbr)
    zs2, _ = o.product()
    # the program orders the Chebyshev terms by record position (k = it - 1): its sum is
    # the accumulator times exp(i acos Es), the same |zS2prod|^2
    phase = np.exp(1j * np.arccos((etot - run.emindlt) / run.delta2))
    assert np.abs(z - zs2 * phase).max() <= 1e-12 * np.abs(zs2).max()
    assert np.allclose(np.abs(z) ** 2, np.abs(zs2) ** 2, rtol=1e-11, atol=1e-14 * np.abs(zs2).max() ** 2)
    # the program's own hbar literal scales the sum by its ratio to the computed one
    z_lit = distri.chebyshev_sum(rec, etot, run.emindlt, run.delta2)
    assert np.allclose(z_lit, z * (distri.HBR / C.hbr), rtol=1e-12, atol=1e-14 * np.abs(zs2).max())


def test_missing_records_are_an_error(tmp_path):
    contfiles.write_cvj_file(str(tmp_path / "Cvjprod.0001"), range(1, 4), np.zeros((3, 1, 2, 2)))
    with pytest.raises(ValueError, match="not complete"):
        distri.read_records(str(tmp_path), 1, 5, (1, 2, 2))
    # a missing later file ends the series (the program's err= branch)
    assert distri.read_records(str(tmp_path), 3, 3, (1, 2, 2)).shape == (3, 1, 2, 2)


def test_packet_distribution_is_smatini_cols(runs):
    run = runs["tiny_j0"]
    i = run.inp
    ft = Oracle(run).flux_tables()
    e = ft["etot"]
    paq, pini = distri.packet_distribution(e, i.rmis2, i.rfin2, i.rcolini_ang, i.ecol_ev, i.deltae_ev, run.xm2reac,
                                           i.Jtot, i.jref, i.iomref, hbr=C.hbr, npunt=1000)
    both = (ft["apaqini"] > 1e-10) & (paq > 1e-10)
    assert both.sum() > len(e) // 2
    assert np.allclose(paq[both], ft["apaqini"][both], rtol=1e-9)
    # the program's own grid (1024 points) and rounded hbar literal (which enters the
    # packet's k0 and width) move it by ~1e-4 relative
    p2, _ = distri.packet_distribution(e, i.rmis2, i.rfin2, i.rcolini_ang, i.ecol_ev, i.deltae_ev, run.xm2reac,
                                       i.Jtot, i.jref, i.iomref)
    assert np.allclose(p2[both], paq[both], rtol=1e-3)


def loops(zs2, fac, j0, om0, photonorm):
    """distriwvp.f:487-525 as written."""
    nom, nj, nv, ne = zs2.shape
    vibrot = np.zeros((nv, ne, nj))
    vibprod = np.zeros((nv, ne))
    s2no = np.zeros(ne)
    for ie in range(ne):
        for iv in range(nv):
            vr = np.zeros(nj)
            for io in range(nom):
                iom = om0 + io
                rot = np.zeros(nj)
                if abs(iom) <= j0 + nj - 1:
                    for jj in range(max(abs(iom), j0) - j0, nj):
                        zzz = zs2[io, jj, iv, ie] / 2.0 / math.pi
                        s = (zzz * zzz.conjugate()).real * fac[ie, iv, jj]
                        s2no[ie] += s
                        vibprod[iv, ie] += s
                        rot[jj] += s
                        vr[jj] += rot[jj]
            vibrot[iv, ie] = vr * photonorm
    return vibrot, vibprod * photonorm, s2no * photonorm


def test_distribution_tables():
    rng = np.random.default_rng(5)
    zs2 = rng.standard_normal((3, 4, 2, 6)) + 1j * rng.standard_normal((3, 4, 2, 6))
    fac = rng.uniform(0.0, 2.0, (6, 2, 4))
    got = distri.distributions(zs2, fac, 1, 0, photonorm=0.7)
    want = loops(zs2, fac, 1, 0, 0.7)
    for a, b in zip(got, want):
        assert np.allclose(a, b, rtol=1e-13, atol=0)


def test_program_on_a_case(runs, case_dirs, tmp_path):
    run = runs["tiny_j3"]
    case = case_dirs["tiny_j3"]
    pp, o, rows = oracle_history(run, 20)
    g = namelist.read(os.path.join(case, "input.dat"))
    g["inputprod"] = dict(iprod=2, nviniprod=pp.nviniprod, nvmaxprod=pp.nvmaxprod, jiniprod=pp.jiniprod,
                          jmaxprod=pp.jmaxprod, iomminprod=pp.iomminprod, iommaxprod=pp.iommaxprod,
                          rbalinprod=3.0, n2prod0=pp.n2prod0, n2prod1=pp.n2prod1, nangproj0=pp.nangproj0,
                          nangproj1=pp.nangproj1)
    g["inputtime"] = dict(g["inputtime"], ntimes=10, nloop=2)
    rundir = tmp_path / "J003"
    rundir.mkdir()
    (rundir / "input.dat").write_text(namelist.dumps(g))
    contfiles.write_cvj_file(str(rundir / "Cvjprod.0001"), range(1, 11), rows[:10])
    contfiles.write_cvj_file(str(rundir / "Cvjprod.0002"), range(11, 21), rows[10:])
    njp, nvp = pp.jmaxprod - pp.jiniprod + 1, pp.nvmaxprod - pp.nviniprod + 1
    # product levels on func/bcwf's absolute scale: around the reactant reference level
    i = run.inp
    eref_raw = distri._bcwf_energy(os.path.join(case, "func", "bcwf"), i.npun1, i.jini, i.nvini, i.nvref, i.jref,
                                   i.ielecref)
    ediatprod = eref_raw + 0.05 * np.arange(njp * nvp, dtype=np.float64).reshape(njp, nvp) - 0.3
    funcdir = tmp_path / "func_copy"
    potini.write_prodwf(str(tmp_path / "prod"), pp.jiniprod, pp.nviniprod, np.zeros((njp, nvp, 1, pp.n2prod1)),
                        ediatprod, pp.nobcprod)
    funcdir.mkdir()
    for name in ("bcwf", "eref"):
        (funcdir / name).write_text(open(os.path.join(case, "func", name)).read())
    (funcdir / "prodwf").write_text(open(str(tmp_path / "prod" / "func" / "prodwf")).read())
    e, vibrot, vibprod, s2no = distri.run_program(str(rundir), potdir=os.path.join(case, "pot"),
                                                  funcdir=str(funcdir))
    assert vibrot.shape == (nvp, run.inp.netot, njp) and np.all(vibrot >= 0) and s2no.max() > 0
    lines = open(str(rundir / ("distriS2prod.v%02d.e1" % pp.nviniprod))).read().splitlines()
    assert len(lines) == run.inp.netot and len(lines[0].split()) == 1 + njp
    vib = np.loadtxt(str(rundir / "distriS2prod.vib"))
    assert vib.shape == (run.inp.netot, 2 + nvp)
    assert np.allclose(vib[:, 1], s2no, rtol=1e-6)


def test_photodissociation_branch(runs, case_dirs, tmp_path):
    """iphoto > 0: S2prodfac = 4 pfin / (pi mu') with no packet distribution, and
    every table scaled by photonorm from the auto file (distriwvp.f:320-327, 436-438)."""
    from madwave3_gb300 import photo
    e = np.array([0.5, 1.0, 2.0])
    ed = np.array([[0.2, 1.5]])                        # [v][j]
    fac = distri.s2prodfac(e, ed, 0.1, 1500.0, iphoto=1)
    ekf = e[:, None, None] - ed[None] + 0.1
    want = np.where(ekf > 0, 4.0 * np.sqrt(np.maximum(ekf, 0) * 1500.0 * 2.0) / distri.HBR / (math.pi * 1500.0), 0.0)
    assert np.allclose(fac, want, rtol=1e-14)
    assert fac[0, 0, 1] == 0.0                          # closed channel
    # the program reads photonorm from the wave's auto file
    run = runs["tiny_j3"]
    case = case_dirs["tiny_j3"]
    pp, o, rows = oracle_history(run, 10)
    g = namelist.read(os.path.join(case, "input.dat"))
    g["inputprod"] = dict(iprod=2, nviniprod=pp.nviniprod, nvmaxprod=pp.nvmaxprod, jiniprod=pp.jiniprod,
                          jmaxprod=pp.jmaxprod, iomminprod=pp.iomminprod, iommaxprod=pp.iommaxprod,
                          rbalinprod=3.0, n2prod0=pp.n2prod0, n2prod1=pp.n2prod1, nangproj0=pp.nangproj0,
                          nangproj1=pp.nangproj1)
    g["inputprocess"] = dict(iphoto=1)
    g["inputtime"] = dict(g["inputtime"], ntimes=10, nloop=1)
    out = {}
    for name, norm in (("a", 1.0), ("b", 0.25)):
        rundir = tmp_path / name
        rundir.mkdir()
        (rundir / "input.dat").write_text(namelist.dumps(g))
        contfiles.write_cvj_file(str(rundir / "Cvjprod.0001"), range(2, 12), rows)
        i = run.inp
        photo.write_auto_file(str(rundir / ("auto.v%02d.j%02d.J%03d" % (i.nvref, i.jref, i.Jtot))), norm, -0.1,
                              run.emindlt, run.delta2, [1], [0.5])
        njp, nvp = pp.jmaxprod - pp.jiniprod + 1, pp.nvmaxprod - pp.nviniprod + 1
        eref_raw = distri._bcwf_energy(os.path.join(case, "func", "bcwf"), i.npun1, i.jini, i.nvini, i.nvref,
                                       i.jref, i.ielecref)
        potini.write_prodwf(str(tmp_path / ("p" + name)), pp.jiniprod, pp.nviniprod,
                            np.zeros((njp, nvp, 1, pp.n2prod1)), np.full((njp, nvp), eref_raw - 0.2), pp.nobcprod)
        fdir = tmp_path / ("f" + name)
        fdir.mkdir()
        (fdir / "bcwf").write_text(open(os.path.join(case, "func", "bcwf")).read())
        (fdir / "prodwf").write_text(open(str(tmp_path / ("p" + name) / "func" / "prodwf")).read())
        out[name] = distri.run_program(str(rundir), potdir=os.path.join(case, "pot"), funcdir=str(fdir))
    assert out["a"][3].max() > 0
    assert np.allclose(out["b"][3], 0.25 * out["a"][3], rtol=1e-14)


def test_distri_reproduces_printprob(runs):
    """The main program's product total S2no (printprob, from the propagation's
    zS2prod accumulators and ini_transcoor's S2prodfac) and distriwvp's, rebuilt
    from the per-iteration Cvjprod records with its own packet distribution and
    hbar literal, agree to the latter's ~1e-4 differences."""
    from madwave3_gb300 import printprob
    from madwave3_gb300.host import transcoor
    run = runs["tiny_j3"]
    i = run.inp
    pp, o, rows = oracle_history(run, 60)
    ft = o.flux_tables()
    etot = ft["etot"]
    njp, nvp = pp.jmaxprod - pp.jiniprod + 1, pp.nvmaxprod - pp.nviniprod + 1
    ediatprod = -0.3 + 0.07 * np.arange(njp * nvp, dtype=np.float64).reshape(njp, nvp)   # zot, from eref
    fac_main = transcoor.s2prodfac(run, etot, ft["apaqini"], ediatprod, pp.nobcprod, pp.nviniprod, pp.nvmaxprod)
    zs2, _ = o.product()
    s2no_main, _ = printprob.s2prod_products(zs2, fac_main, pp)
    z = distri.chebyshev_sum(rows, etot, run.emindlt, run.delta2)
    paq, pini = distri.packet_distribution(etot, i.rmis2, i.rfin2, i.rcolini_ang, i.ecol_ev, i.deltae_ev,
                                           run.xm2reac, i.Jtot, i.jref, i.iomref)
    fac_d = distri.s2prodfac(etot, ediatprod.T, 0.0, run.xm2prod, paq, pini, run.xm2reac)
    _, _, s2no_d = distri.distributions(z, fac_d, pp.jiniprod, pp.iomminprod)
    big = s2no_main > 1e-3 * s2no_main.max()
    assert big.sum() > 10
    assert np.allclose(s2no_d[big], s2no_main[big], rtol=1e-3)
