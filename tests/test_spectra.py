"""cheby-spectra (SRC/photo/cheby-spectra.f) restated: the auto file the
photodissociation path writes, read back, and the damped Chebyshev transform
checked on autocorrelations whose spectrum is known in closed form."""
import math

import numpy as np
import pytest

from madwave3_gb300 import photo, spectra

EMINDLT, DELTA2 = 1.0, 2.0          # zots: Es = (E - 1) / 2


def zot_to_ev(e):
    return e / (spectra.CONVE1 * spectra.EV2CM)


def one_state(es0, k):
    """<psi0| T_k(H_s) |psi0> of a packet that is one eigenstate at scaled energy es0."""
    return np.cos(np.arange(k + 1) * math.acos(es0))


def run(auto, ne=8001, xkgam=4e-3, es_lo=-0.95, es_hi=0.95, xnorm=0.37, ebnd=-0.2, eref=0.05):
    lo, hi = zot_to_ev(EMINDLT + es_lo * DELTA2), zot_to_ev(EMINDLT + es_hi * DELTA2)
    return spectra.spectrum(auto, xnorm, ebnd, EMINDLT, DELTA2, eref, lo, hi, ne, xkgam)


def test_auto_file_round_trip(tmp_path):
    p = str(tmp_path / "auto.v00.j00.J001")
    autos = [0.5, -0.25, 1.0e-300, 3.5e-7]
    photo.write_auto_file(p, 0.397, -0.123456789, 9.44, 9.87, [1, 2, 3, 4], autos)
    xnorm, eb, em, d2, auto = spectra.read_auto_file(p)
    assert (xnorm, eb, em, d2) == pytest.approx((0.397, -0.123456789, 9.44, 9.87), rel=1e-11)
    assert auto[0] == 1.0 and np.allclose(auto[1:], autos, rtol=1e-15, atol=0)
    # the program reads at most kmax lines
    assert len(spectra.read_auto_file(p, kmax=2)[4]) == 3


def test_one_state_peak_and_norm():
    es0 = 0.25
    sp = run(one_state(es0, 5000))
    e0 = zot_to_ev(EMINDLT + es0 * DELTA2)
    step = sp["E_ev"][1] - sp["E_ev"][0]
    assert abs(sp["E_ev"][np.argmax(sp["spectrum_au"])] - e0) <= step
    # the transform of one state is a normalised peak (Lorentzian tails beyond the
    # grid's ends are the small remainder)
    assert sp["integral"] == pytest.approx(1.0, abs=0.01)


def test_two_states_split_the_norm():
    w1, es1, es2 = 0.3, -0.4, 0.5
    auto = w1 * one_state(es1, 5000) + (1.0 - w1) * one_state(es2, 5000)
    sp = run(auto)
    assert sp["integral"] == pytest.approx(1.0, abs=0.01)
    e = sp["E_ev"]
    mid = zot_to_ev(EMINDLT + 0.05 * DELTA2)
    step = e[1] - e[0]
    below = float(np.sum(sp["spectrum_au"][e < mid])) / 0.37 * step / spectra.AU2EV
    assert below == pytest.approx(w1, abs=0.01)


def test_outside_the_chebyshev_range_is_zero():
    """|Es| > 1 is 0 (the program's isnan test); the grid avoids |Es| = 1 itself,
    where the program divides by zero and writes an infinity."""
    sp = run(one_state(0.1, 200), es_lo=-1.5, es_hi=1.5, ne=300)
    es = (sp["E_ev"] * spectra.EV2CM * spectra.CONVE1 - EMINDLT) / DELTA2
    assert np.all(np.isfinite(sp["spectrum"]))
    assert np.all(sp["spectrum"][np.abs(es) > 1.0] == 0.0)
    assert np.any(sp["spectrum"][np.abs(es) < 1.0] != 0.0)


def test_units_of_the_table():
    """Photon energy and cross section as the program forms them (:88-96)."""
    sp = run(one_state(0.25, 400), ne=101, xnorm=0.5, ebnd=-0.3, eref=0.2)
    eshift = 0.2 / (spectra.CONVE1 * spectra.EV2CM)
    assert np.allclose(sp["ephoton_au"], (sp["E_ev"] + eshift + 0.3) / spectra.AU2EV, rtol=1e-15)
    assert np.allclose(sp["xsection_au"], sp["ephoton_au"] * sp["spectrum_au"] / (137.0 * 0.07957747),
                       rtol=1e-14)
    assert np.allclose(sp["spectrum_au"], sp["spectrum"] / (math.pi * spectra.HBR * spectra.ZOT2AU), rtol=1e-14)


def test_command_line(tmp_path):
    a = str(tmp_path / "auto")
    photo.write_auto_file(a, 0.4, -0.1, EMINDLT, DELTA2, range(1, 301), one_state(0.2, 300)[1:])
    eref = tmp_path / "eref"
    eref.write_text("0.0\n")
    out = str(tmp_path / "spec")
    spectra.main([a, "--eref-file", str(eref), "--emin", "0.5", "--emax", "1.5", "--ne", "11", "--xkgam",
                  "0.01", "--out", out])
    lines = open(out).read().splitlines()
    assert len(lines) == 12 and lines[-1].startswith("  integral=")
    assert len(lines[0].split()) == 6
