"""Precision gate of the mixed form: |Delta P(E)| of the mixed path against the
FP64 path after a full propagation of a workload.

    python -m madwave3_gb300.gate --case j0_256x128x60 --iterations 2000 [--out FILE]

Both runs start from the same packet and take the same number of Chebyshev
iterations; P(E) is the total reaction probability of totalflux
(SRC/mod_flux_01y2.f:778-816).  Prints one JSON line with max |Delta P|, the
energy where it occurs, max P, the iterations and both paths' wall times.
"""
import argparse
import json
import os
import tempfile
import time

import numpy as np


def run_gate(case, iterations, cases_dir=None, waves=None):
    from . import Propagator
    from .host import generator, setup

    base = cases_dir or os.path.join(tempfile.gettempdir(), "mw3_gate_cases")
    d = os.path.join(base, case)
    if not os.path.exists(os.path.join(d, "pot", "cont.pot")):
        generator.write_case(d, **generator.CASES[case])
    run = setup.load(os.path.join(d, "input.dat"))
    out = {"case": case, "iterations": iterations, "stored_points": int(run.ntot)}
    res = {}
    for prec in ("fp64", "mixed"):
        p = Propagator(run, prec)
        p.start()
        p.sync()
        t = time.time()
        p.run(iterations - 1)
        p.sync()
        out["seconds_" + prec] = time.time() - t
        res[prec] = p.totalflux()[0]
        res[prec + "_norm"] = p.norms()[-1]
        p.close()
    a, b = res["fp64"], res["mixed"]
    e = np.linspace(run.inp.ekinmin_ev, run.inp.ekinmax_ev, run.inp.netot)
    k = int(np.argmax(np.abs(a - b)))
    out.update({"max_abs_dP": float(np.abs(a - b).max()), "at_energy_ev": float(e[k]),
                "max_P": float(np.abs(a).max()), "mean_P": float(np.mean(a)),
                "final_norm_fp64": float(res["fp64_norm"]), "final_norm_mixed": float(res["mixed_norm"]),
                "pass_1e-4": bool(np.abs(a - b).max() <= 1e-4)})
    return out, e, a, b


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="j0_256x128x60")
    ap.add_argument("--iterations", type=int, default=2000)
    ap.add_argument("--out", default=None, help="also write E, P_fp64, P_mixed as text")
    args = ap.parse_args()
    out, e, a, b = run_gate(args.case, args.iterations)
    if args.out:
        np.savetxt(args.out, np.stack([e, a, b], 1), header="E(eV) P_fp64 P_mixed")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
