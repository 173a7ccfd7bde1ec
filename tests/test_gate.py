"""Host arithmetic of the precision gate: the energy window of the state-resolved
comparison and the per-channel table (no GPU)."""
import types

import numpy as np

from madwave3_gb300 import gate


def _run(nvini=0, jini=0, netot=5):
    inp = types.SimpleNamespace(nvini=nvini, jini=jini, netot=netot, ekinmin_ev=0.1, ekinmax_ev=0.5)
    return types.SimpleNamespace(inp=inp)


def test_energy_window_keeps_the_packets_energies():
    a = np.array([1e-9, 1e-3, 0.5, 1.0, 2e-4])
    w = gate.energy_window(a)
    assert w.tolist() == [False, True, True, True, False]
    assert gate.energy_window(np.zeros(3)).all()


def test_vj_error_and_channel_table_inside_the_window():
    run = _run(nvini=0, jini=1)
    a = np.zeros((2, 2, 5))
    b = np.zeros((2, 2, 5))
    a[0, 1] = [0.1, 0.2, 0.3, 0.2, 9.0]
    b[0, 1] = [0.1, 0.2, 0.31, 0.2, 1.0]          # the big difference lies outside the window
    a[1, 0] = [0.0, 0.5, 0.5, 0.5, 0.0]
    b[1, 0] = a[1, 0] + 1e-6
    w = np.array([True, True, True, True, False])
    e = gate._vj_error(run, a, b, w)
    assert np.isclose(e["max_abs_dP_vj"], 0.01)
    assert (e["at_v"], e["at_j"]) == (1, 1)
    assert np.isclose(e["at_energy_ev_vj"], 0.3)
    assert np.isclose(e["max_P_vj"], 0.5)
    assert e["vj_window_ev"] == [0.1, 0.4]
    rows = gate.channel_table(run, a, b, w)
    assert [r[:2] for r in rows] == [[1, 1], [0, 2]]
    assert np.isclose(rows[0][2], 0.01) and np.isclose(rows[0][3], 0.3)
    assert np.isclose(rows[1][2], 1e-6) and np.isclose(rows[1][3], 0.5)
