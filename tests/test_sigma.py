"""sigmaFromS2prod's cross section (SRC/AUXILIARy-CODES/sigmaFromS2prod.f)
from per-J probabilities: the partial-wave sum and the J-shifting rules."""
import math

import numpy as np

from madwave3_gb300 import sigma


def _calc(js, f, e):
    return {J: (e, f(e)) for J in js}


def test_flat_probabilities_sum_to_the_partial_wave_formula():
    e = sigma.ev_to_au(np.linspace(0.1, 1.5, 60))
    grid = sigma.energy_grid(0.2, 1.4, 25)
    pj = sigma.jshift_pj(_calc(range(0, 11), lambda x: np.full_like(x, 0.3), e), {}, 10, grid)
    assert np.allclose(pj, 0.3, atol=1e-12)
    s = sigma.cross_section({0: pj}, grid, 2.014, 1.008, 1.008, iprod=0)
    mu = 1.008 * (2.014 + 1.008) / (2.014 + 1.008 + 1.008) * sigma.CONVM
    expect = math.pi / (2 * mu * grid) * 0.3 * 11 ** 2 * sigma.CONVL ** 2
    assert np.allclose(s, expect, rtol=1e-12)


def test_j_shifting_between_and_beyond_the_calculated_j():
    e = sigma.ev_to_au(np.linspace(0.05, 2.0, 400))
    f = lambda x: 0.5 * (1 + np.tanh((x - sigma.ev_to_au(0.6)) / sigma.ev_to_au(0.05)))
    be = {0: sigma.ev_to_au(0.002), 4: sigma.ev_to_au(0.002)}
    grid = sigma.energy_grid(0.3, 1.2, 40)
    pj = sigma.jshift_pj(_calc([0, 4], f, e), be, 6, grid)
    # J = 1: (3/4) P_0 shifted by 2 B + (1/4) P_4 shifted by -18 B
    b = be[0]
    want = 0.75 * f(grid - b * 2) + 0.25 * f(grid - b * (2 - 20))
    assert np.max(np.abs(pj[:, 1] - want)) < 2e-3
    # J = 6 > 4: P_4 shifted by B (42 - 20)
    assert np.max(np.abs(pj[:, 6] - f(grid - b * 22))) < 2e-3
    assert np.max(np.abs(pj[:, 4] - f(grid))) < 2e-3


def test_reads_the_probability_files(tmp_path):
    from madwave3_gb300.printprob import e17_7e3
    p = tmp_path / "S2prod"
    with open(p, "w") as fh:
        for x, y in ((0.1, 0.2), (0.5, 1.0000001), (0.9, 0.4)):
            fh.write("".join(" " + e17_7e3(v) for v in (x, y, y + 0.1, 0.0)) + "\n")
    e, pj, pp = sigma.read_pj(str(p))
    assert np.allclose(e, sigma.ev_to_au(np.array([0.1, 0.5, 0.9])))
    assert pj[1] == 1.0 and np.all(pp == 0)
