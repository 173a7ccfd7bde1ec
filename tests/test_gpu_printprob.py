"""printprob's S2prod / S2prodelec from the GPU's FP64 accumulators against the
same files from the oracle's, after the same iterations."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["tiny_j3", "tiny_e2"])
def test_gpu_s2prod_matches_oracle(runs, case, tmp_path):
    from madwave3_gb300 import Propagator, printprob
    from oracle.mw3ref import Oracle

    run = runs[case]
    os.makedirs(str(tmp_path / "o"))
    os.makedirs(str(tmp_path / "g"))
    o = Oracle(run)
    o.start(run.psi0)
    o.run_iters(70)
    zs2o, _ = o.s2()
    ft = o.flux_tables()
    po = printprob.write_s2prod(str(tmp_path / "o"), run, 1, *o.totalflux(), zs2o, ft["etot"], ft["reacfct"],
                                o.s2factor())
    p = Propagator(run, "fp64")
    p.start()
    p.run(70)
    tb = p.tables()
    printprob.write_s2prod(str(tmp_path / "g"), run, 1, *p.totalflux(), p.accumulators()["zs2"], tb["etot"],
                                tb["reacfct"], tb["s2factor"])
    p.close()
    for name in (os.path.basename(po), "S2prodelec"):
        a = printprob.read_s2prod(str(tmp_path / "g" / name))
        b = printprob.read_s2prod(str(tmp_path / "o" / name))
        # the FP64 paths agree to ~1e-12; printed with 7 digits a value may round
        # differently in its last digit
        np.testing.assert_allclose(a, b, rtol=1.01e-6, atol=1e-300)
