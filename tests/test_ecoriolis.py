"""The electronic Coriolis variant of H psi (mod_Hphi_eCoriolis_01y2.f) in the
oracle, checked against a direct numpy restatement of its one extra term.

The variant differs from the plain difs only by a j^2-type coupling between
channels of equal Omega whose diatomic Lambda differ by one (angkinj2
:186-324, difs :901-911).  tiny_ecor has two states, Lambda = 0 and 1, same
sigma, J = 2, Omega = 0..2.
"""
import math

import numpy as np
import pytest

from madwave3_gb300.host import constants as C
from oracle.mw3ref import Oracle


@pytest.fixture(scope="module")
def ecor_run(runs):
    return runs["tiny_ecor"]


def ecor_pairs(run):
    """(source, target) channel pairs the variant couples: equal Omega, equal
    sigma, |Lambda - Lambda'| = 1."""
    out = []
    for b in range(run.ncan):
        for b2 in range(run.ncan):
            e, e2 = run.nelebas[b] - 1, run.nelebas[b2] - 1
            if b == b2 or run.iombas[b] != run.iombas[b2] or run.sigdiat[e] != run.sigdiat[e2]:
                continue
            if abs(int(run.iomdiat[e]) - int(run.iomdiat[e2])) == 1:
                out.append((b, b2))
    return out


def ecor_matrix(run, b, b2):
    """X[ir1, i, j] = sum_k y_k(r1) D_b(i, j_k) D_b(j, j_k) over the basis
    indices k at which both channels hold the same j (angkinj2 :249-285)."""
    i = run.inp
    na, n1 = i.nangu, i.npun1
    e, e2 = run.nelebas[b] - 1, run.nelebas[b2] - 1
    lam, lam2 = int(run.iomdiat[e]), int(run.iomdiat[e2])
    r1 = i.rmis1 + run.ah1 * np.arange(n1)
    X = np.zeros((n1, na, na))
    jjjmax = (na - 1) * i.inc
    for k in range(min(run.nojbas[b], run.nojbas[b2])):
        j = int(run.jbas[b, k])
        if j != int(run.jbas[b2, k]) or j > jjjmax:
            continue
        xk = math.sqrt(lam * lam + lam2 * lam2) * math.sqrt(j * (j + 1) - abs(lam * lam2)) * C.hbr * C.hbr
        if lam == 0 or lam2 == 0:
            xk *= math.sqrt(2.0)
        y = np.minimum(xk / (run.xm1red * r1 * r1), run.rotcutmax)
        d = run.djmmp[run.iombas[b], e, j, :]
        X += y[:, None, None] * d[None, :, None] * d[None, None, :]
    return X


def ecor_term(run, psi):
    """The variant's extra contribution to H psi, from the rectangles of psi."""
    i = run.inp
    na, n1, n2 = i.nangu, i.npun1, i.npun2
    rect = np.zeros((run.ncan, na, n1, n2))
    for iang in range(1, na + 1):
        n = run.npunreal[iang - 1]
        r1, r2 = run.indr1[iang - 1, :n] - 1, run.indr2[iang - 1, :n] - 1
        for b in range(run.ncan):
            o = run.offs[iang - 1, b]
            rect[b, iang - 1, r1, r2] = psi[o:o + n]
    out = np.zeros(run.ntot)
    for b, b2 in ecor_pairs(run):
        X = ecor_matrix(run, b, b2)
        for iang in range(1, na + 1):
            n = run.npunreal[iang - 1]
            r1, r2 = run.indr1[iang - 1, :n] - 1, run.indr2[iang - 1, :n] - 1
            o = run.offs[iang - 1, b2]
            src = rect[b][:, r1, r2]                    # [jang, point]
            out[o:o + n] += np.einsum("jp,pj->p", src, X[r1, iang - 1, :])
    return out


def test_case_has_coupled_channels(ecor_run):
    run = ecor_run
    assert list(run.iomdiat) == [0, 1] and run.sigdiat[0] == run.sigdiat[1]
    pairs = ecor_pairs(run)
    # Omega = 0, 1, 2 each hold a Lambda = 0 and a Lambda = 1 channel
    assert len(pairs) == 6
    # Omega = 0: the Lambda = 1 basis starts at j = 1, so no basis index k holds
    # the same j in both channels and the coupling vanishes (the k-th entries are
    # compared, angkinj2 :246-251); Omega = 1 and 2 couple
    for b, b2 in pairs:
        X = ecor_matrix(run, b, b2)
        if run.iombas[b] == 0:
            assert not X.any()
        else:
            assert np.abs(X).max() > 0


def test_three_states_give_two_sources(runs):
    run = runs["tiny_ecor3"]
    assert list(run.iomdiat) == [0, 1, 0]
    targets = {}
    for b, b2 in ecor_pairs(run):
        targets.setdefault(b2, []).append(b)
    # every Lambda = 1 channel takes both Lambda = 0 channels of its Omega
    lam1 = [b for b in range(run.ncan) if run.iomdiat[run.nelebas[b] - 1] == 1]
    assert lam1 and all(len(targets[b]) == 2 for b in lam1)


@pytest.mark.parametrize("case", ["tiny_ecor", "tiny_ecor3"])
def test_oracle_term_matches_restatement(runs, case):
    run = runs[case]
    plain, ecor = Oracle(run), Oracle(run, ecoriolis=True)
    rng = np.random.default_rng(20261204)
    for _ in range(2):
        psi = rng.uniform(-1, 1, run.ntot)
        d = ecor.hphi(psi) - plain.hphi(psi)
        want = ecor_term(run, psi)
        assert np.abs(want).max() > 1e-3 * np.abs(plain.hphi(psi)).max()
        assert np.abs(d - want).max() <= 1e-12 * np.abs(want).max()


def test_equal_lambda_leaves_h_unchanged(runs):
    """All states Lambda = 0: the variant's H is the plain one, bit for bit."""
    run = runs["tiny_e2"]
    psi = np.random.default_rng(7).uniform(-1, 1, run.ntot)
    assert np.array_equal(Oracle(run).hphi(psi), Oracle(run, ecoriolis=True).hphi(psi))


def test_threaded_oracle_agrees(ecor_run):
    run = ecor_run
    psi = np.random.default_rng(3).uniform(-1, 1, run.ntot)
    one = Oracle(run, ecoriolis=True).hphi(psi)
    four = Oracle(run, ecoriolis=True, threads=4).hphi(psi)
    assert np.abs(one - four).max() <= 1e-13 * np.abs(one).max()
