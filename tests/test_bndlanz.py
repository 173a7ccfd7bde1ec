"""Lanczos bound states (SRC/bound-lanz): the recursion, the Cullum-Willoughby
selection of true eigenvalues, the conjugate-gradient eigenvectors and the
initial guess, on CPU with the oracle's H psi as the operator (the GPU's
H psi against it is in test_gpu_bndlanz.py)."""
import numpy as np
import pytest

from madwave3_gb300 import bndlanz
from madwave3_gb300.host.constants import ev_to_zot, zot_to_ev


def test_true_eigenvalues_of_a_known_spectrum():
    """300 Lanczos steps on a 30-dimensional operator: T has 301 Ritz values
    (many ghost copies); valnkry's selection keeps each of the 30 once."""
    rng = np.random.default_rng(20261203)
    d = np.sort(rng.uniform(-1, 1, 30))
    v1 = rng.uniform(-1, 1, 30)
    v1 /= np.linalg.norm(v1)
    et, a, b = bndlanz.lanczos_eigenvalues(lambda x: d * x, v1, nkrymax=300, ntimes=100)
    assert a.size == 301                       # the last block overshoots nkrymax as the reference does
    assert et.size == 30
    assert np.max(np.abs(et - d)) < 1e-8


def test_selection_rules():
    """Multiple copies are true even when T-hat (T without its first row and
    column) has them; a simple value that T-hat also has is spurious."""
    # T = [[5, .3, 0], [.3, 1, 0], [0, 0, 2]]: 2 is simple and in T-hat -> spurious;
    # the two eigenvalues of the coupled 2 x 2 block are not in T-hat -> true
    et = bndlanz.converged_eigenvalues([5.0, 1.0, 2.0], [0.3, 0.0])
    assert np.allclose(et, np.linalg.eigvalsh([[5.0, 0.3], [0.3, 1.0]]), atol=1e-14)
    # T = diag(5, 2, 2): 2 twice -> true once; 5 simple and in T-hat -> spurious
    et = bndlanz.converged_eigenvalues([5.0, 2.0, 2.0], [0.0, 0.0])
    assert np.allclose(et, [2.0])


@pytest.fixture(scope="module")
def tiny(runs):
    from oracle.mw3ref import Oracle
    run = runs["tiny_j0"]
    return run, Oracle(run)


def test_initial_vector(tiny):
    run, _ = tiny
    emax = run.vmintot + ev_to_zot(1.0)
    v = bndlanz.initial_vector(run, emax)
    assert abs(np.dot(v, v) - 1.0) < 1e-14
    nz = v > 0
    assert 0 < nz.sum() < run.ntot
    assert np.allclose(v[nz], v[nz][0])
    with pytest.raises(ValueError):
        bndlanz.initial_vector(run, run.vmintot - 1.0)


def test_lanczos_matches_a_direct_eigensolver(tiny):
    from scipy.sparse.linalg import LinearOperator, eigsh
    run, o = tiny
    v1 = bndlanz.initial_vector(run, run.vmintot + ev_to_zot(1.0))
    et, a, b = bndlanz.lanczos_eigenvalues(o.hphi, v1, nkrymax=400, ntimes=200)
    A = LinearOperator((run.ntot, run.ntot), matvec=o.hphi, dtype=np.float64)
    w = np.sort(eigsh(A, k=4, which="SA", tol=1e-12)[0])
    assert np.max(np.abs(et[:4] - w)) < 1e-10


def test_cg_eigenvectors(tiny):
    from scipy.sparse.linalg import LinearOperator, eigsh
    run, o = tiny
    bs = bndlanz.BoundStates(run, o.hphi, zot_to_ev(run.vmintot) + 1.0, ntimes=200, nkrymax=400,
                             criter_ev=1e-6, nomxiter=3000, nvecmax=2)
    bs.eigenvalues()
    A = LinearOperator((run.ntot, run.ntot), matvec=o.hphi, dtype=np.float64)
    w, V = eigsh(A, k=2, which="SA", tol=1e-12)
    for k, (e, v, em, its, ok) in enumerate(bs.eigenvectors()):
        assert ok
        assert abs(em - e) <= bs.criter
        assert abs(np.dot(v, V[:, k])) > 0.9999


def test_levels_file(tmp_path):
    p = tmp_path / "niveles.dat"
    bndlanz.write_levels(str(p), [-0.0123456789, 0.5, 3.0], vcutmax=2.0)
    lines = p.read_text().splitlines()
    assert len(lines) == 2
    assert lines[0] == "     1   -0.1234568E-01   -0.1031385E+03   -0.1278761E-01"
    assert bndlanz._e15(0.5) == "  0.5000000E+00"
    assert bndlanz._e15(123.45678) == "  0.1234568E+03"
    assert bndlanz._e15(0.99999999) == "  0.1000000E+01"


def test_bound_state_files_and_the_photodissociation_start(tiny, tmp_path):
    """write_bnd's files, read back by dip_bndgrid's mapping (iphoto = 2) on the
    same grid, give the bound state itself as the initial packet, which then
    propagates."""
    run, o = tiny
    bs = bndlanz.BoundStates(run, o.hphi, zot_to_ev(run.vmintot) + 1.0, ntimes=200, nkrymax=400,
                             criter_ev=1e-6, nomxiter=3000, nvecmax=1)
    bs.eigenvalues()
    e, v, em, its, ok = bs.eigenvectors()[0]
    bndlanz.write_bnd(str(tmp_path), run, 1, e, v)
    lines = (tmp_path / "grid.ip000").read_text().splitlines()
    assert int(lines[0]) == run.ntot and len(lines) == 4 + run.ntot
    assert len(lines[4]) == 9 * 8
    psi0, e_ev, nrm = bndlanz.initial_from_bound(run, str(tmp_path), 1)
    assert np.allclose(psi0, v, rtol=0, atol=1e-15)
    assert abs(e_ev - zot_to_ev(e)) < 1e-12 and abs(nrm - 1.0) < 1e-12
    o.start(psi0)
    o.run_iters(5)
    assert np.all(np.isfinite(o.state()[1]))


def test_assignment_distributions(tiny):
    """bndassign: for a state on a single (angle, R) line the v distribution is
    the squared overlap with each diatomic function; populations of Omega and
    of the electronic states add up to the norm."""
    from madwave3_gb300.host import generator

    run, _ = tiny
    blk, ang, r1, r2 = run.point_table()
    line = (blk == 0) & (ang == ang[0]) & (r2 == r2[0])
    rng = np.random.default_rng(5)
    v = np.zeros(run.ntot)
    v[line] = rng.standard_normal(line.sum())
    v /= np.linalg.norm(v)
    fdp, _, _ = generator.product_states(run, 30, 0, 0, 0, 2, **generator.CASES["tiny_j0"])
    a = bndlanz.assign(run, v, fdprod=fdp[0])
    e = run.nelebas[0] - 1
    for k in range(a["disv1"].size):
        want = np.dot(run.fd[e, 0, k, r1[line] - 1], v[line]) ** 2
        assert abs(a["disv1"][k] - want) < 1e-14
    assert a["disv2"].shape == (3,) and np.all(a["disv2"] >= 0)
    assert abs(sum(a["disomg"].values()) - 1.0) < 1e-12
    assert abs(a["diselec"].sum() - 1.0) < 1e-12
    assert abs(a["cos_mean"] - run.cgamma[ang[0] - 1]) < 1e-12


def _blocks(path, ncol=3):
    """Blank-line separated blocks of a plot file, as arrays."""
    out, cur = [], []
    for line in open(path).read().split("\n"):
        if line.strip():
            cur.append([float(x) for x in line.split()])
        elif cur:
            out.append(np.array(cur))
            cur = []
    return out


def test_plot_bnd_files(runs, tmp_path):
    """plot_bnd's three files (main_boundlanz.f:620-811) on a seeded vector."""
    import math
    run = runs["tiny_j3"]
    i = run.inp
    vec = np.random.default_rng(17).standard_normal(run.ntot)
    bndlanz.plot_bnd(str(tmp_path), run, 4, vec)
    tot = float(np.sum(vec * vec))
    lab = bndlanz._point_labels(run)
    # summed over r1 (per R and angle) and over angles (per R and r1): each block an R
    a = _blocks(str(tmp_path / "bndplot.i004"))
    b = _blocks(str(tmp_path / "bndr1r2.i004"))
    assert len(a) == i.npun2 and all(x.shape == (i.nangu, 3) for x in a)
    assert len(b) == i.npun2 and all(x.shape == (i.npun1, 3) for x in b)
    assert abs(sum(x[:, 2].sum() for x in a) - tot) <= 1e-6 * tot
    assert abs(sum(x[:, 2].sum() for x in b) - tot) <= 1e-6 * tot
    for jr2 in (0, i.npun2 // 2):
        want = float(np.sum(vec[lab[:, 6] == jr2 + 1] ** 2))
        assert abs(a[jr2][:, 2].sum() - want) <= 1e-6 * max(want, 1e-300)
    assert np.allclose(a[0][:, 1], np.arccos(run.cgamma[: i.nangu]), rtol=1e-6)
    # the bond cut: one block per x1, each value psi (not squared) of a stored point
    # at that r1, or 0
    c = _blocks(str(tmp_path / "bndbondx1x2.i004"))
    assert len(c) == i.npun1 and all(x.shape == (i.npun1, 3) for x in c)
    nonzero = 0
    for jr1, blk in enumerate(c):
        at = vec[lab[:, 5] == jr1 + 1]
        for v in blk[:, 2]:
            if v != 0.0:
                nonzero += 1
                assert np.min(np.abs(at - v)) <= 1e-6 * abs(v)
    assert nonzero > 0
    xb = math.cos(135.5 * math.pi / 180.0)
    assert np.allclose(c[3][:, 0], i.rmis1 + 3 * run.ah1, rtol=1e-6) and xb < 0
