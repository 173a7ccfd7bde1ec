"""Product diatom states of uncoupled electronic states (the diabatic_prod_pot
= 0 branch of product_radialf_write, bndbc1ele) on Morse potentials, whose
levels are known in closed form, and the func/prodwf file they are written to."""
import math
import os
from types import SimpleNamespace

import numpy as np

from madwave3_gb300.host import constants as C
from madwave3_gb300.host import potini, setup

A, RE = 1.03, 1.4                           # bohr^-1, bohr
MORSE = [(0.17, 0.0), (0.12, 0.02)]         # (De, asymptote) of each state, hartree
MU = 918.6                                  # a.u.


def potelebond(r1, r2, ctet):
    v = np.zeros((len(MORSE), len(MORSE), len(r2)))
    for k, (de, top) in enumerate(MORSE):
        v[k, k] = de * (1.0 - np.exp(-A * (r2 - RE))) ** 2 - de + top
    return v


def morse_level(k, v):
    de, top = MORSE[k]
    w = A * math.sqrt(2.0 * de / MU)
    return top - de + w * (v + 0.5) - w * w / (4.0 * de) * (v + 0.5) ** 2


def grid(n2prod1=600):
    rmis2, rfin2 = 0.1 * C.convl, 15.0 * C.convl            # angstrom
    g = SimpleNamespace(inp=SimpleNamespace(rmis2=rmis2, rfin2=rfin2, npun2=1024), xm1prod=MU / C.convm)
    g.ah2 = (rfin2 - rmis2) / 1023.0
    return g, n2prod1


def test_levels_order_and_normalisation():
    g, n2p = grid()
    fd, e, nob, elec, vib = potini.product_radialf_write_adiabatic(
        g, potelebond, 0, 7, 0, 0, n2p, nelec=2, max_viblevels=[5, 3])
    # state 1's five levels, then state 2's three, in that order (not sorted by energy)
    assert nob[0] == 7
    assert list(elec[0]) == [1] * 5 + [2] * 3 and list(vib[0]) == [0, 1, 2, 3, 4, 0, 1, 2]
    want = [morse_level(0, v) for v in range(5)] + [morse_level(1, v) for v in range(3)]
    got = e[0] / C.conve1 * C.conve                         # zot -> hartree
    assert np.allclose(got, want, rtol=1e-6, atol=0)
    # each function lives in its own state and is discrete-normalised
    for k in range(8):
        own = elec[0, k] - 1
        assert abs(np.sum(fd[0, k, own] ** 2) - 1.0) < 1e-10
        assert not fd[0, k, 1 - own].any()


def test_rotation_raises_the_levels_and_nvini_numbers():
    g, n2p = grid()
    _, e0, _, _, _ = potini.product_radialf_write_adiabatic(g, potelebond, 0, 3, 0, 4, n2p)
    assert np.all(np.diff(e0[:, 0]) > 0)                   # v = 0 rises with j
    _, e1, nob1, _, vib1 = potini.product_radialf_write_adiabatic(g, potelebond, 1, 3, 0, 0, n2p,
                                                                  max_viblevels=[4])
    # the count starts at nvini - 1, so nvini numbers the state's v = 0 (nothing is
    # skipped); of its four levels the fourth, numbered 4 > nvmaxprod, is dropped
    assert list(vib1[0]) == [0, 1, 2] and np.allclose(e1[0], e0[0, :3], rtol=1e-12) and nob1[0] == 3


def test_prodwf_file_round_trip(tmp_path):
    g, n2p = grid(200)
    fd, e, nob, elec, vib = potini.product_radialf_write_adiabatic(
        g, potelebond, 0, 5, 0, 1, n2p, nelec=2, max_viblevels=[4, 2])
    potini.write_prodwf(str(tmp_path), 0, 0, fd, e, nob, elec, vib)
    f2, e2, n2, el2, vb2 = setup.product_radialf_read(os.path.join(str(tmp_path), "func", "prodwf"), 0, 1, 0, 5, n2p,
                                                      eref=0.25)
    assert np.array_equal(n2, nob) and np.array_equal(el2, elec) and np.array_equal(vb2, vib)
    assert np.array_equal(f2, fd) and np.allclose(e2, e - 0.25, rtol=0, atol=1e-15)
