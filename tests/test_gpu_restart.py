"""Stop and resume through the continuation files: a fresh context that reads
contNN.paq / contNN.S2 (mw3_upload_state_all, mw3_upload_accumulators) and
runs on gives the same numbers as the run that never stopped."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_continuation_through_cont_files(runs, precision, tmp_path):
    from madwave3_gb300 import Propagator, contfiles

    run = runs["tiny_j3"]
    a = Propagator(run, precision)
    a.start()
    a.run(50)
    km1, k, it = a.state_all()
    acc = a.accumulators()
    contfiles.write_cont(str(tmp_path), km1, k, acc["zs2"], acc["zcr"], acc["zcdr"], iit0=it, indt=0, iloop=1)
    a.run(45)
    ref = (a.state_all()[1], a.totalflux()[0], a.accumulators())
    a.close()

    r = contfiles.read_cont(str(tmp_path), zs2_shape=acc["zs2"].shape, flux_shape=acc["zcr"].shape)
    b = Propagator(run, precision)
    b.upload_state_all(r["psi_km1"], r["psi_k"], r["iit0"])
    b.upload_accumulators(0, r["zcr"], r["zcdr"], r["zs2"])
    b.run(45)
    got = (b.state_all()[1], b.totalflux()[0], b.accumulators())
    b.close()
    # the same launches on the same data: equal bits are expected; the bar
    # allows for a zero's sign in the FP32 ring sums, nothing more
    def same(a, b):
        return np.max(np.abs(a - b)) <= 1e-13 * max(np.max(np.abs(b)), 1e-300)

    assert same(got[0], ref[0])
    assert same(got[1], ref[1])
    for key in ("zcr", "zcdr", "zs2", "cvj"):
        assert same(got[2][key], ref[2][key]), key
