"""The photodissociation workload: three diabatic states started from the
lowest bound state of the ground surface times a constant transition dipole.

The reference's photodissociation run is three programs on one grid:
``bndgrid.out`` computes the bound states of the initial electronic state
(SRC/bound-lanz/main_boundlanz.f, stored with write_bnd), ``pot.out`` writes
the transition dipole on the grid (set_trans_dipole), and ``mad3.out`` builds
the initial packet from them (dip_bnd / dip_bndgrid) and propagates it.
``photodissociation`` runs the same chain on the synthetic surfaces of
``host/generator.py``:

1. the bound-state case: the ground diabatic surface alone (one electronic
   state), total angular momentum ``jtotini`` with the parity opposite to the
   final states' (a dipole transition changes it), on the final case's grid;
2. Lanczos on it through the library's FP64 H psi (``nlanczos`` steps), the
   lowest eigenvalue, its eigenvector by conjugate gradients, written with
   write_bnd;
3. the final case (``nelecmax`` states, iphoto = 1) and the packet
   d.e |bound> with a constant dipole ``dipole_au`` along z for every final
   state (madwave3_gb300.photo), renormalised, photonorm kept.

Needs the GPU (the Lanczos steps call mw3_hphi).
"""
import os

import numpy as np

from . import bndlanz, photo
from .host import generator, setup


def _ensure_case(d, params):
    if not os.path.exists(os.path.join(d, "pot", "cont.pot")):
        generator.write_case(d, **params)


def photodissociation(base, case="e3_384x192x80", jtotini=1, nlanczos=100, dipole_au=1.0, emax_lanzini_ev=1.0,
                      cg_iterations=200):
    """Returns the final run with its initial packet in ``run.psi0`` and the
    packet's norm before renormalisation in ``run.photonorm``, and a summary
    (bound-state energy, Lanczos and CG details, Omega populations)."""
    from .propagator import Propagator

    final = dict(generator.CASES[case])
    final["iphoto"] = 1
    ipar_final = final.get("iparity", generator.DEFAULT["iparity"])
    bound = dict(generator.CASES[case])
    bound.update(nelecmax=1, Jtot=jtotini, iommin=0, iommax=jtotini, iparity=-ipar_final, iphoto=0)
    dfin = os.path.join(base, case + "_photo")
    dbnd = os.path.join(base, case + "_bound_J%d" % jtotini)
    _ensure_case(dfin, final)
    _ensure_case(dbnd, bound)
    rb = setup.load(os.path.join(dbnd, "input.dat"))
    summary = {"jtotini": jtotini, "iparini": -ipar_final, "nlanczos": nlanczos, "bound_blocks": int(rb.ncan)}
    if not os.path.exists(os.path.join(dbnd, "bnd.iv000.ip000")):
        pb = Propagator(rb, "fp64")
        v1 = bndlanz.initial_vector(rb, emax_lanzini_ev * generator.C.eV2cm * generator.C.conve1)
        etrue, alpha, beta = bndlanz.lanczos_eigenvalues(pb.hphi, v1, nkrymax=nlanczos, ntimes=nlanczos)
        if len(etrue):
            e0 = float(etrue[0])
        else:           # no copy confirmed within the steps: the lowest Ritz value
            from scipy.linalg import eigh_tridiagonal
            e0 = float(eigh_tridiagonal(alpha, beta[: len(alpha) - 1], eigvals_only=True)[0])
        vec, emean, its, ok = bndlanz.cg_eigenvector(pb.hphi, v1, e0, cg_iterations, 1e-6)
        pb.close()
        vec = vec / np.linalg.norm(vec)
        bndlanz.write_bnd(dbnd, rb, 0, e0, vec)
        summary.update(lanczos_true=int(len(etrue)), cg_iterations=int(its), cg_converged=bool(ok))
    rf = setup.load(os.path.join(dfin, "input.dat"))
    dip = photo.dipole_table(rf, lambda r, R, c: (0.0, 0.0, dipole_au))
    psi0, pnorm, e_ev, per_om = photo.initial_packet(rf, dbnd, 0, 1, Jtotini=jtotini, iparini=-ipar_final,
                                                    dipol=dip)
    rf.psi0 = psi0
    rf.photonorm = pnorm
    summary.update(bound_energy_ev=e_ev, photonorm=pnorm, omega_populations=per_om, stored_points=int(rf.ntot),
                   blocks=int(rf.ncan))
    return rf, summary
