"""Photodissociation start on the host (SRC/mod_photoini_01y2.f): 3j symbols,
the transition-operator coefficients, the dipole files and the dipole-weighted
initial packet, and the autocorrelation file."""
import math
import os

import numpy as np
import pytest

from madwave3_gb300 import photo


def test_threej_known_values_and_orthogonality():
    assert photo.threej(1, 1, 0, 0, 0, 0) == pytest.approx(-1.0 / math.sqrt(3.0), abs=1e-15)
    assert photo.threej(1, 1, 1, 1, -1, 0) == pytest.approx(1.0 / math.sqrt(6.0), abs=1e-15)
    assert photo.threej(2, 1, 1, 0, 0, 0) == pytest.approx(math.sqrt(2.0 / 15.0), abs=1e-15)
    assert photo.threej(1, 1, 1, 0, 0, 0) == 0.0                      # odd sum of j with all m = 0
    assert photo.threej(1, 1, 3, 0, 0, 0) == 0.0                      # outside the triangle
    for j1, j2 in ((2, 1), (3, 2)):
        for j3 in range(abs(j1 - j2), j1 + j2 + 1):
            for j3p in range(abs(j1 - j2), j1 + j2 + 1):
                m3 = 0
                s = sum(photo.threej(j1, j2, j3, m1, -m1 - m3, m3) * photo.threej(j1, j2, j3p, m1, -m1 - m3, m3)
                        for m1 in range(-j1, j1 + 1) if abs(m1 + m3) <= j2)
                assert s == pytest.approx((1.0 / (2 * j3 + 1)) if j3 == j3p else 0.0, abs=1e-14)


def test_factresj():
    """dip_bnd's coefficients: zero when the parities are equal, and for
    Jini = 0 -> J = 1 only Omega_ini = 0 contributes."""
    assert not np.any(photo.factresj(1, 1, 0, 1))
    f = photo.factresj(1, -1, 0, 1)
    assert np.any(np.abs(f) > 1e-10)
    assert not np.any(f[1:])
    # |<00 1q|1 Omega>|: the two q = 0 / Omega = 0 and q = 1 / Omega = 1 entries
    assert abs(f[0, 1, 0]) > 0 and abs(f[0, 2, 1]) > 0


@pytest.fixture(scope="module")
def photo_runs(case_dirs):
    """J = 0 (+ parity) and J = 1 (- parity) on the two-state grid."""
    import copy
    from madwave3_gb300.host import generator, setup
    r0, r1 = setup.load_sweep(os.path.join(case_dirs["tiny_e2"], "input.dat"), [0, 1], generator.jsweep_inputs)
    r1 = copy.copy(r1)
    r1.inp = copy.copy(r1.inp)
    r1.inp.iphoto = 1
    return r0, r1


def test_dipole_files_round_trip(photo_runs, tmp_path):
    _, run = photo_runs
    dip = photo.dipole_table(run, lambda r, R, c: (0.1 * r, 0.0, 1.0 + 0.01 * R * c))
    assert dip.shape == (run.inp.nangu, run.npuntot, run.nelec, 3)
    n = run.npunreal[0]
    assert np.allclose(dip[0, :n, :, 1], dip[0, :n, :, 1][:, :1])        # d_0 = d_z, the same for both states
    assert np.allclose(dip[0, :n, :, 0], -dip[0, :n, :, 2])               # d_{-1} = -d_{+1}
    photo.write_dipole_files(str(tmp_path), run, dip)
    back = photo.read_dipole_files(str(tmp_path), run)
    for a in range(run.inp.nangu):
        m = run.npunreal[a]
        assert np.array_equal(back[a, :m], dip[a, :m])


def test_initial_packet_from_a_stored_bound_state(photo_runs, tmp_path):
    """iphoto = 1 from a bound state of J = 0 written by write_bnd: unit norm,
    photonorm = |d.e psi|^2, only Omega' = 0, 1 (|q| <= 1), and iphoto = 2 of
    the same state reproduces it on the J = 0 run itself."""
    from madwave3_gb300 import bndlanz
    r0, r1 = photo_runs
    rng = np.random.default_rng(3)
    vec = rng.standard_normal(r0.ntot)
    vec /= np.linalg.norm(vec)
    bndlanz.write_bnd(str(tmp_path), r0, 0, -0.01, vec)
    dip = photo.dipole_table(r1, lambda r, R, c: (0.0, 0.0, 1.0))
    psi0, pnorm, e_ev, per_om = photo.initial_packet(r1, str(tmp_path), 0, 1, Jtotini=0, iparini=1, dipol=dip)
    assert abs(np.dot(psi0, psi0) - 1.0) < 1e-12
    assert pnorm > 0 and abs(sum(per_om.values()) - 1.0) < 1e-12
    from madwave3_gb300.host.constants import zot_to_ev
    assert abs(e_ev - zot_to_ev(-0.01)) < 1e-15           # write_bnd takes zot, stores eV
    # a constant d_z couples Omega_ini = 0 to Omega = 0 only (q = 0)
    assert per_om.get(1, 0.0) < 1e-20 and per_om[0] == pytest.approx(1.0)
    # iphoto = 2 with one bound electronic state: the state's ielec = 1 part, renormalised
    p2, n2, _, _ = photo.initial_packet(r0, str(tmp_path), 0, 2)
    first = bndlanz._point_labels(r0)[:, 1] == 1
    ref = np.where(first, vec, 0.0)
    assert abs(n2 - np.dot(ref, ref)) < 1e-14
    assert np.allclose(p2, ref / np.linalg.norm(ref), rtol=0, atol=1e-15)


def test_auto_file(tmp_path):
    p = str(tmp_path / "auto.v00.j00.J001")
    photo.write_auto_file(p, 0.5, -0.25, 9.5, 9.7, [1, 2], [1.0, 0.25])
    lines = open(p).read().splitlines()
    head = lines[0].split()
    assert len(head) == 4 and head[0] == "0.500000000000D+00" and head[1] == "-0.250000000000D+00"
    assert [float(x.replace("D", "E")) for x in head] == [0.5, -0.25, 9.5, 9.7]
    assert lines[1].split() == ["1", "1.0"] and lines[2].split() == ["2", "0.25"]
