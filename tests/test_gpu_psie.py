"""funE (SRC/mod_PsiE_01y2.f:92-123): psi(E) accumulated on the device every
iteration at the energies of &inputPsiE, against the oracle."""
import numpy as np
import pytest

from madwave3_gb300.host import constants as C

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("case", ["tiny_j0", "tiny_e2"])
def test_zfe_against_the_oracle(runs, case):
    import copy
    from madwave3_gb300 import Propagator
    from oracle.mw3ref import Oracle

    run = copy.copy(runs[case])
    energies_ev = [0.3, 0.55, 0.9]
    run.efe_zot = np.array(energies_ev) * C.eV2cm * C.conve1
    ref = Oracle(run, nofe_energies_ev=energies_ev)
    ref.start(run.psi0)
    ref.run_iters(60)
    zr = ref.zfe()
    assert np.abs(zr).max() > 0
    out = {}
    for prec in ("fp64", "mixed"):
        p = Propagator(run, prec)
        p.start()
        p.run(60)
        out[prec] = p.psi_e()
        p.close()
    assert out["fp64"].shape == zr.shape == (3, run.ntot)
    assert rel(out["fp64"], zr) < 1e-10
    assert rel(out["mixed"], zr) < 1e-4
