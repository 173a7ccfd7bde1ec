"""Parity pinned to the reference's own numbers: the shipped H + HD run.

EXAMPLES/HD+H_collision/J000-check holds the log (sal.000) and probability
file of a J = 0 run of the reference on its neural-network H3 surface.  The
restated pot.out (madwave3_gb300/host/potini.py, h3nn.py) tabulates that
surface from the example's input file; the host set-up and the CPU oracle
then have to reproduce what the reference printed: every reactant diatomic
level (17 digits), the stored points of each of the run's 7 processes, the
potential minimum, the initial packet's norm and mean energy (one H psi),
and the start of the norm trace ||psi_k||^2.  The GPU path is checked
against the whole trace and P(E) in test_gpu_example.py."""
import os

import numpy as np

from madwave3_gb300.host import constants as C


def test_reactant_levels(example_case, example_pins):
    """ediat(v, j) - ediatref for every (j, v) the log lists (sal.000:346-549),
    including the j = 37..39 entries that the run's level counts of 0 left at
    ediat = 0."""
    _, s = example_case
    ev = (s["ediat"] - s["ediatref"]) / C.conve1 / C.eV2cm
    rows = example_pins["reactant_levels_ev"]
    assert len(rows) == 203
    listed = set()
    for ie, j, v, e in rows:
        assert abs(ev[ie - 1, j, v] - e) < 1e-12, (j, v, ev[ie - 1, j, v], e)
        listed.add((j, v))
    # and nothing the log does not list
    nobc = s["nobc"][0]
    assert {(j, v) for j in range(nobc.size) for v in range(nobc[j] + 1)} == listed


def test_stored_points_per_process(example_case, example_pins):
    """ntotproc of the 7-process run (sal.000:793-799): process p holds the
    angles nangu - p, nangu - p - 7, ... (paralelizacion's round robin)."""
    _, s = example_case
    npr = s["npunreal"]
    nproc = len(example_pins["ntotproc"])
    per = [0] * nproc
    for iang in range(1, npr.size + 1):
        per[(npr.size - iang) % nproc] += int(npr[iang - 1])
    assert per == example_pins["ntotproc"]
    assert sum(per) == 704278


def test_potential_minimum(example_case, example_pins):
    _, s = example_case
    assert abs(s["vmin"] / C.conve1 / C.eV2cm - example_pins["vmin_ev"]) < 1e-14


def test_initial_packet_norm(example_run, example_pins):
    """'Norm of initial wavepacket' (sal.000:856): the packet on the compressed
    grid with the Numerov v = 0, j = 0 function of the surface."""
    n = float(np.sum(example_run.psi0 ** 2))
    assert abs(n - example_pins["initial_norm"]) < 1e-13


def test_oracle_mean_energy_and_norm_trace(example_run, example_pins):
    """The oracle's H psi_0 gives the printed mean energy <psi_0|H|psi_0>
    (sal.000:1156), and its first 20 Chebyshev iterations the printed
    ||psi_k||^2, k = 2..21 (sal.000:1160+): agreement at the 1e-12 level, the
    rest being the summation order of the 7 processes and of the DSTs."""
    from oracle.mw3ref import Oracle
    run = example_run
    o = Oracle(run, threads=os.cpu_count() or 1)
    h = o.hphi(run.psi0)
    em = float(np.dot(run.psi0, h)) / C.conve1 / 8065.5
    assert abs(em - example_pins["mean_energy_ev"]) / example_pins["mean_energy_ev"] < 1e-13
    o.start(run.psi0)
    n = o.run_iters(20)
    ref = np.array(example_pins["norm_trace"][1:21])
    assert np.max(np.abs(n - ref) / ref) < 5e-12


def _product_setup(example_case, example_run):
    _, s = example_case
    return s["product"]


def test_product_levels(example_case, example_run, example_pins):
    """ediatprod(v, j) - ediatref of the product diatom (sal.000:561-791): the
    box DVR of the diabatic product branch, all 21 x 11 levels."""
    fd, ed, nob = _product_setup(example_case, example_run)
    ev = (ed - example_run.ediatref) / C.conve1 / C.eV2cm
    rows = example_pins["product_levels_ev"]
    assert len(rows) == 231 and np.all(nob == 10)
    for j, v, e in rows:
        assert abs(ev[j, v] - e) < 1e-12, (j, v, ev[j, v], e)


def test_product_projection_tables(example_case, example_run, example_pins):
    """ini_transcoor on the example: transRgjac's sum of squares over process
    0's angles (the log's xt1, sal.000:1143), the sampled product distances
    (rpbmin, rpbmax) and the norm of every product state's projection function
    (sal.000:909-1139, printed to 7 digits)."""
    from madwave3_gb300.host import transcoor
    run = example_run
    fd, ed, nob = _product_setup(example_case, example_run)
    tr = transcoor.trans_rg_jac(run, 6.0, 1, run.inp.nangu)
    _, ang, _, _ = run.point_table()
    xt1 = float(np.sum(tr[ang % 7 == 0] ** 2))
    assert abs(xt1 - 7372.9687214579890) / 7372.9687214579890 < 1e-13
    _, rpb, _, _, ok = transcoor.prod_geometry(run, 6.0, 1, run.inp.npun2, 1, run.inp.nangu)
    assert abs(rpb[ok].min() - 4.6465921805298308e-2) < 1e-15
    assert abs(rpb[ok].max() - 24.752987568936842) < 1e-13
    wf = transcoor.prod_functions_omega(run, 6.0, fd, nob, 0, 20, 0, 1, run.inp.npun2, 1, run.inp.nangu, 0)
    rows = example_pins["product_wf_norms"]
    assert len(rows) == 231
    for iom, j, v, n in rows:
        x = float(np.sum(wf[j, v] ** 2))
        assert abs(x - n) <= 5e-7 * n, (j, v, x, n)


def test_oracle_flux_gate_switch(runs):
    """The oracle's totalflux_k with and without the E > V(flux point) test
    (SRC/mod_flux_01y2.f:640): for each flux point and energy above the point's
    potential the two forms hold the same sums; below it the gated form holds
    0 and the gate-free form the point's contribution."""
    from oracle.mw3ref import Oracle
    run = runs["tiny_j0"]
    i = run.inp
    out = []
    for gate in (True, False):
        o = Oracle(run, flux_gate=gate)
        o.start(run.psi0)
        o.run_iters(30)
        out.append(o.flux()[0])
    etot = Oracle(run).flux_tables()["etot"]
    poti = []                        # the flux points in the reference's order: angle, block, point
    for iang in run.angle_order():
        n = run.npunreal[iang - 1]
        ir1 = run.indr1[iang - 1, :n]
        r1 = i.rmis1 + (ir1 - 1) * run.ah1
        ir1f = ir1[r1 <= i.r1flux_ang].max()
        for b in range(run.ncan):
            e = run.nelebas[b] - 1
            poti.extend(run.vvv[e, e, iang - 1, :n][ir1 == ir1f])
    poti = np.array(poti)
    zg, zn = out
    assert zg.shape == zn.shape == (poti.size, etot.size)
    above = etot[None, :] > poti[:, None]
    assert above.any() and (~above).any()
    assert np.array_equal(zg[above], zn[above])
    assert np.all(zg[~above] == 0) and np.any(zn[~above] != 0)
