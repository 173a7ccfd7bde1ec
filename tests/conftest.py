import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (run on the GB300)")


@pytest.fixture(scope="session")
def case_dirs(tmp_path_factory):
    """The small generated cases the oracle finishes in seconds."""
    from madwave3_gb300.host import generator
    base = tmp_path_factory.mktemp("cases")
    out = {}
    for name in ("tiny_j0", "tiny_j3", "tiny_e2", "tiny_ecor", "tiny_ecor3"):
        d = str(base / name)
        generator.write_case(d, **generator.CASES[name])
        out[name] = d
    return out


@pytest.fixture(scope="session")
def runs(case_dirs):
    from madwave3_gb300.host import setup
    return {k: setup.load(os.path.join(d, "input.dat")) for k, d in case_dirs.items()}


def synthetic_product_tables(run, seed=20261203):
    """Seeded product-projection tables for a generated case (the parity of
    prodpaq / prodcvj is pure arithmetic on whatever ini_transcoor produced)."""
    import numpy as np
    from madwave3_gb300.product import ProductProjection

    rng = np.random.default_rng(seed)
    i = run.inp
    n2p0, n2p1 = 3, max(3, i.npun2 - 4)
    a0, a1 = 2, max(2, i.nangu - 1)
    om0, om1 = 0, min(2, i.Jtot)
    jp0, jp1 = 0, 5
    vp0, vp1 = 0, 2
    nobc = rng.integers(vp0, vp1 + 1, size=jp1 - jp0 + 1).astype(np.int32)
    nom, njp, nvp = om1 - om0 + 1, jp1 - jp0 + 1, vp1 - vp0 + 1
    nang, n2p = a1 - a0 + 1, n2p1 - n2p0 + 1
    return ProductProjection(
        n2p0, n2p1, a0, a1, om0, om1, jp0, jp1, vp0, vp1, nobc,
        rng.uniform(0.5, 1.5, run.ntot),
        rng.uniform(-1.0, 1.0, (run.ncan, nom, nang, n2p)),
        rng.standard_normal((nom, njp, nvp, run.nelec, nang, n2p)))


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="session")
def example_pins():
    import json
    with open(os.path.join(GOLDEN, "example_pins.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def example_case(tmp_path_factory, example_pins):
    """The reference's shipped H + HD example (EXAMPLES/HD+H_collision: J = 0,
    256 r1 x 256 R x 140 angles, its neural-network H3 surface), tabulated by
    the restated pot.out from the example's input file and the surface's
    weights (tests/golden/).  Returns (case directory, pot.out summary)."""
    from madwave3_gb300.host import h3nn, potini
    d = str(tmp_path_factory.mktemp("example") / "HD+H")
    nn = h3nn.H3NN(os.path.join(GOLDEN, "h3nn_weights.json"))
    summary = potini.write_case(d, None, nn.potelebond, bound_test="below_asymptote",
                                input_text=example_pins["input_dat"])
    return d, summary


@pytest.fixture(scope="session")
def example_run(example_case):
    from madwave3_gb300.host import setup
    return setup.load(os.path.join(example_case[0], "input.dat"))
