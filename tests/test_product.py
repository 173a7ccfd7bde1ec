"""The oracle's prodpaq / prodcvj (SRC/mod_coortrans01_02.f:694-825) against a
numpy restatement of the same sums, on seeded tables (no reference test or
golden vector covers the product projection: parity unpinned beyond this)."""
import numpy as np

from conftest import synthetic_product_tables


def numpy_cvjprod(run, pp, psi):
    i = run.inp
    nom, njp, nvp = pp.shape
    nang, n2p = pp.nangproj1 - pp.nangproj0 + 1, pp.n2prod1 - pp.n2prod0 + 1
    fun = np.zeros((run.ncan, nang, n2p))
    for b in range(run.ncan):
        for iang in range(pp.nangproj0, pp.nangproj1 + 1):
            o = run.offs[iang - 1, b]
            n = run.npunreal[iang - 1]
            ir2 = run.indr2[iang - 1, :n]
            w = pp.transrgjac[o:o + n] * psi[o:o + n]
            sel = (ir2 >= pp.n2prod0) & (ir2 <= pp.n2prod1)
            np.add.at(fun[b, iang - pp.nangproj0], ir2[sel] - pp.n2prod0, w[sel])
    cvj = np.zeros((nom, njp, nvp))
    for b in range(run.ncan):
        e = run.nelebas[b] - 1
        for o in range(nom):
            aux2 = fun[b] * pp.dtrans[b, o]
            for jj in range(max(0, pp.iomminprod + o - pp.jiniprod), njp):
                for vv in range(pp.nobcprod[jj] - pp.nviniprod + 1):
                    cvj[o, jj, vv] += np.sum(pp.prodwf[o, jj, vv, e] * aux2)
    return cvj


def test_oracle_product_projection(runs):
    from oracle.mw3ref import Oracle

    run = runs["tiny_j3"]
    pp = synthetic_product_tables(run)
    o = Oracle(run)
    o.set_product(pp)
    o.start(run.psi0)
    zs2 = np.zeros(pp.shape + (run.inp.netot,), complex)
    for k in range(12):
        o.run_iters(1)
        _, psi, it = o.state()
        cvj = numpy_cvjprod(run, pp, psi)
        zs2 += cvj[..., None] * o.coefecheby(it)[None, None, None, :]
    z, c = o.product()
    assert np.max(np.abs(c - cvj)) < 1e-12 * np.max(np.abs(cvj))
    assert np.max(np.abs(z - zs2)) < 1e-12 * np.max(np.abs(zs2))
    # rows outside j >= max(jiniprod, Omega), v <= noBCprod(j) stay zero
    assert np.all(z[cvj == 0] == 0)
