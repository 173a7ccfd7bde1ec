"""CUDA-graph replay of 32-iteration blocks against the same iterations launched
one kernel at a time (MW3_NO_GRAPHS=1): the wave packets, norms and every
accumulator agree bit for bit, across blocks that start on either psi buffer,
calls that end mid-block, and the elastic channel gated below kminelastic."""
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _trajectory(run, precision, monkeypatch, graphs):
    from madwave3_gb300 import Propagator

    monkeypatch.setenv("MW3_NO_GRAPHS", "0" if graphs else "1")
    p = Propagator(run, precision)
    p.start()
    l0 = p.kernel_launches()
    out = []
    for n in (100, 70, 45):             # 3 blocks + 4 eager, 28 eager + 1 block + 10, ...
        p.run(n)
        out.append(p.state()[1].copy())
    runs = run if isinstance(run, list) else [run]
    for w in range(len(runs)):
        out.append(p.norms(w))
        out.append(p.totalflux(w)[0])
        acc = p.accumulators(w)
        out.extend(acc[k] for k in sorted(acc))
    launches = p.kernel_launches() - l0
    p.close()
    return out, launches


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("case", ["tiny_j0", "tiny_j3", "tiny_e2"])
def test_graph_replay_matches_eager(runs, case, precision, monkeypatch):
    eager, n_eager = _trajectory(runs[case], precision, monkeypatch, False)
    graph, n_graph = _trajectory(runs[case], precision, monkeypatch, True)
    assert len(eager) == len(graph)
    for a, b in zip(eager, graph):
        assert np.array_equal(np.asarray(a), np.asarray(b))
    # every kernel of a replayed block is counted, plus the one that sets its base
    assert n_eager <= n_graph <= n_eager + 215 // 32 + 1


def test_graph_replay_two_waves(runs, monkeypatch):
    both = [runs["tiny_j0"], runs["tiny_j3"]]
    eager, _ = _trajectory(both, "mixed", monkeypatch, False)
    graph, _ = _trajectory(both, "mixed", monkeypatch, True)
    for a, b in zip(eager, graph):
        assert np.array_equal(np.asarray(a), np.asarray(b))


def test_graph_replay_with_elastic_gate(monkeypatch):
    """kminelastic = 50: the blocks that would cross the gate run eagerly."""
    from madwave3_gb300.host import generator, setup

    with tempfile.TemporaryDirectory() as d:
        generator.write_case(d, **dict(generator.CASES["tiny_j3"], kminelastic=50))
        run = setup.load(os.path.join(d, "input.dat"))
    eager, _ = _trajectory(run, "mixed", monkeypatch, False)
    graph, _ = _trajectory(run, "mixed", monkeypatch, True)
    for a, b in zip(eager, graph):
        assert np.array_equal(np.asarray(a), np.asarray(b))
