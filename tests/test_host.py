"""Host-side set-up mirror and input generator (no GPU)."""
import os

import numpy as np
import pytest

from madwave3_gb300.host import generator, namelist, setup


def test_namelist_reads_reference_style_input(tmp_path):
    text = """&INPUTGRIDBASE
 NPUN1=    256, RMIS1=     0.1d0     , RFIN1=  20.d0     , NPUN1MIN= 64,
 NANGU= 140,  JTOT=     0, IPARITY=  1
 /
&inputpotmass
!-----------> masses
system='H+DH'
xm0=2.014101779d0
/
"""
    g = namelist.parse(text)
    assert g["inputgridbase"]["npun1"] == 256 and g["inputgridbase"]["rfin1"] == 20.0
    assert g["inputpotmass"]["system"] == "H+DH" and g["inputpotmass"]["xm0"] == 2.014101779
    again = namelist.parse(namelist.dumps(g))
    assert again == g


def test_generated_files_follow_reference_formats(case_dirs):
    d = case_dirs["tiny_e2"]
    lines = open(os.path.join(d, "pot", "cont.pot")).read().split("\n")
    assert int(lines[0]) == 2                       # nelec
    npunreal = [int(x) for x in lines[7].split()]
    assert len(npunreal) == 8
    rows = open(os.path.join(d, "pot", "pot.001.dat")).read().split("\n")
    assert len([r for r in rows if r.strip()]) == npunreal[0]
    assert len(rows[0].split()) == 2 + 2 * 2       # ir1 ir2 ((V(ie,je),ie),je)
    assert os.path.exists(os.path.join(d, "func", "bcwf")) and os.path.exists(os.path.join(d, "func", "eref"))


def test_djmmp_orthonormal(runs):
    for run in runs.values():
        assert setup.check_djmmp(run) < 1e-13


def test_flat_layout(runs):
    run = runs["tiny_j3"]
    blk, ang, r1, r2 = run.point_table()
    assert len(blk) == run.ntot
    # angle-major from nangu down to 1, then block, then point
    first = ang[0]
    assert first == run.inp.nangu and blk[0] == 0
    assert np.all(np.diff(-ang) >= 0)


def test_initial_packet_norm(runs):
    for run in runs.values():
        assert abs(np.sum(run.psi0 ** 2) - run.gauss_norm) < 0.05


def test_parity_rule_and_sweep_block_count():
    """basis drops Omega=0 when iparity differs from sigma (-1)^J; the J=0..40
    sweep with parity (-1)^J keeps it and has 266 blocks."""
    total = 0
    for J in range(41):
        over = generator.jsweep_inputs(J)
        r = setup.Run(inp=setup.Inputs(nangu=10, inc=1, Jtot=J, iparity=over["iparity"], iommin=0,
                                       iommax=over["iommax"], jmax=5))
        r.nelec = 1
        r.iomdiat = np.zeros(1, np.int32); r.iomatom = np.zeros(1, np.int32)
        r.sigdiat = np.ones(1); r.sigatom = np.ones(1)
        r.inp.xm2 = 1.0
        setup.basis(r)
        total += r.ncan
        assert 0 in r.iombas
    assert total == 266
    r = setup.Run(inp=setup.Inputs(nangu=10, inc=1, Jtot=3, iparity=1, iommin=0, iommax=3, jmax=5, xm2=1.0))
    r.nelec = 1
    r.iomdiat = np.zeros(1, np.int32); r.iomatom = np.zeros(1, np.int32)
    r.sigdiat = np.ones(1); r.sigatom = np.ones(1)
    with pytest.raises(ValueError):
        setup.basis(r)                              # Omega=0 dropped: iommin must be 1


def test_truncated_potential_file_is_rejected(case_dirs, tmp_path):
    import shutil
    d = str(tmp_path / "bad")
    shutil.copytree(case_dirs["tiny_j0"], d)
    p = os.path.join(d, "pot", "pot.003.dat")
    rows = open(p).read().split("\n")
    open(p, "w").write("\n".join(rows[: len(rows) // 2]))
    with pytest.raises(ValueError):
        setup.load(os.path.join(d, "input.dat"))


def test_mismatched_grid_is_rejected(case_dirs, tmp_path):
    import shutil
    d = str(tmp_path / "bad2")
    shutil.copytree(case_dirs["tiny_j0"], d)
    g = namelist.read(os.path.join(d, "input.dat"))
    g["inputgridbase"]["npun2"] += 1
    open(os.path.join(d, "input.dat"), "w").write(namelist.dumps(g))
    with pytest.raises(ValueError):
        setup.load(os.path.join(d, "input.dat"))
