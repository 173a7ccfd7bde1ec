"""Precision gate of the mixed form: |Delta P(E)| of the mixed path against the
FP64 path after a full propagation of a workload.

    python -m madwave3_gb300.gate --case j0_256x128x60 --iterations 2000 [--out FILE]
    python -m madwave3_gb300.gate --case j0_256x128x60 --sweep 0,10,20,30,40 --iterations 3000

With --sweep the partial waves J (Omega_max = min(J, 6), parity (-1)^J, the
J = 0..40 sweep's settings) run batched in one context per precision, and the
line reports max |Delta P(E)| for every J.

Both runs start from the same packet and take the same number of Chebyshev
iterations; P(E) is the total reaction probability of totalflux
(SRC/mod_flux_01y2.f:778-816).  Prints one JSON line with max |Delta P|, the
energy where it occurs, max P, the iterations and both paths' wall times, and
the error of the state-resolved probabilities: P_vj(E) of every reactant
channel (v, j), summed over the Omega blocks, as printprob forms them from
zS2 (SRC/main_madwave3.f:640-652), over the energies where the packet's
amplitude |a(E)|^2 is at least 1e-3 of its largest value (S2factor divides by
it, so outside that window both paths' P_vj are rounding over a tiny number).
"""
import argparse
import json
import os
import tempfile
import time

import numpy as np


def state_probabilities(run, prop, wave=0):
    """P[nj][nv][netot]: |S|^2 of every reactant channel (v, j) summed over the
    wave's Omega/electronic blocks (printprob's S2 elements)."""
    from .printprob import s2_elements
    s2 = s2_elements(run, prop.accumulators(wave)["zs2"], prop.tables(wave)["s2factor"])
    return s2.sum(axis=0)


# P_vj(E) carries S2factor's 1/|a(E)|^2 (Smatini_col): where the packet has almost
# no amplitude both paths divide their rounding by a tiny number, so the
# state-resolved comparison covers the energies where |a(E)|^2 is at least this
# fraction of its largest value
VJ_AMPLITUDE_FRACTION = 1e-3


def energy_window(apaqini):
    a = np.asarray(apaqini, np.float64)
    return a >= VJ_AMPLITUDE_FRACTION * a.max() if a.size and a.max() > 0 else np.ones(a.shape, bool)


def _vj_error(run, a, b, window=None):
    d = np.abs(a - b)
    pa = np.abs(a)
    if window is not None:
        d = d * window
        pa = pa * window
    k = np.unravel_index(int(np.argmax(d)), d.shape)
    e = np.linspace(run.inp.ekinmin_ev, run.inp.ekinmax_ev, run.inp.netot)
    out = {"max_abs_dP_vj": float(d.max()), "at_j": int(k[0] + run.inp.jini), "at_v": int(k[1] + run.inp.nvini),
           "at_energy_ev_vj": float(e[k[2]]), "max_P_vj": float(pa.max())}
    if window is not None:
        out["vj_window_ev"] = [float(e[window].min()), float(e[window].max())] if window.any() else None
    return out


def channel_table(run, a, b, window=None, floor=1e-8):
    """One row per reactant channel (v, j) whose P_vj(E) reaches ``floor``
    inside the window: [v, j, max |P_a - P_b|, max P_a] over the energies."""
    w = np.ones(a.shape[-1], bool) if window is None else window
    rows = []
    for jj in range(a.shape[0]):
        for vv in range(a.shape[1]):
            pa, pb = a[jj, vv][w], b[jj, vv][w]
            if pa.size and np.abs(pa).max() >= floor:
                rows.append([int(vv + run.inp.nvini), int(jj + run.inp.jini), float(np.abs(pa - pb).max()),
                             float(np.abs(pa).max())])
    return rows


def run_gate(case, iterations, cases_dir=None, waves=None):
    from .host import generator, setup

    base = cases_dir or os.path.join(tempfile.gettempdir(), "mw3_gate_cases")
    if case.endswith("_photo"):
        from . import workloads
        run, summary = workloads.photodissociation(base, case[: -len("_photo")])
    else:
        d = os.path.join(base, case)
        if not os.path.exists(os.path.join(d, "pot", "cont.pot")):
            generator.write_case(d, **generator.CASES[case])
        run = setup.load(os.path.join(d, "input.dat"))
    return run_gate_run(run, iterations, case)


def run_gate_run(run, iterations, case=""):
    """The gate on one prepared wave (its packet in run.psi0)."""
    from . import Propagator

    out = {"case": case, "iterations": iterations, "stored_points": int(run.ntot)}
    res = {}
    for prec in ("fp64", "mixed"):
        p = Propagator(run, prec)
        p.start([run.psi0])
        p.sync()
        t = time.time()
        p.run(iterations - 1)
        p.sync()
        out["seconds_" + prec] = time.time() - t
        res[prec] = p.totalflux()[0]
        res[prec + "_norm"] = p.norms()[-1]
        res[prec + "_vj"] = state_probabilities(run, p)
        res["window"] = energy_window(p.tables()["apaqini"])
        p.close()
    out.update(_vj_error(run, res["fp64_vj"], res["mixed_vj"], res["window"]))
    a, b = res["fp64"], res["mixed"]
    e = np.linspace(run.inp.ekinmin_ev, run.inp.ekinmax_ev, run.inp.netot)
    k = int(np.argmax(np.abs(a - b)))
    out.update({"max_abs_dP": float(np.abs(a - b).max()), "at_energy_ev": float(e[k]),
                "max_P": float(np.abs(a).max()), "mean_P": float(np.mean(a)),
                "final_norm_fp64": float(res["fp64_norm"]), "final_norm_mixed": float(res["mixed_norm"]),
                "pass_1e-4": bool(np.abs(a - b).max() <= 1e-4)})
    return out, e, a, b


def run_sweep_gate(case, js, iterations, cases_dir=None, channels=False):
    from . import Propagator
    from .host import generator, setup

    base = cases_dir or os.path.join(tempfile.gettempdir(), "mw3_gate_cases")
    d = os.path.join(base, case)
    if not os.path.exists(os.path.join(d, "pot", "cont.pot")):
        generator.write_case(d, **generator.CASES[case])
    runs = setup.load_sweep(os.path.join(d, "input.dat"), js, generator.jsweep_inputs)
    out = {"case": case, "J": list(js), "iterations": iterations,
           "blocks": [int(r.ncan) for r in runs], "stored_points": int(sum(r.ntot for r in runs))}
    res = {}
    for prec in ("fp64", "mixed"):
        p = Propagator(runs, prec)
        p.start()
        p.sync()
        t = time.time()
        p.run(iterations - 1)
        p.sync()
        out["seconds_" + prec] = time.time() - t
        res[prec] = [p.totalflux(w)[0] for w in range(len(runs))]
        res[prec + "_vj"] = [state_probabilities(runs[w], p, w) for w in range(len(runs))]
        res["window"] = [energy_window(p.tables(w)["apaqini"]) for w in range(len(runs))]
        p.close()
    per = []
    for w, J in enumerate(js):
        a, b = res["fp64"][w], res["mixed"][w]
        row = {"J": J, "max_abs_dP": float(np.abs(a - b).max()), "max_P": float(np.abs(a).max())}
        row.update(_vj_error(runs[w], res["fp64_vj"][w], res["mixed_vj"][w], res["window"][w]))
        if channels:
            row["channels"] = channel_table(runs[w], res["fp64_vj"][w], res["mixed_vj"][w], res["window"][w])
        per.append(row)
    out["per_J"] = per
    out["max_abs_dP"] = max(x["max_abs_dP"] for x in per)
    out["max_abs_dP_vj"] = max(x["max_abs_dP_vj"] for x in per)
    out["pass_1e-4"] = bool(out["max_abs_dP"] <= 1e-4)
    out["dst_form"] = "split FP16" if os.environ.get("MW3_DST_TF32", "") != "1" else "3xTF32"
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="j0_256x128x60")
    ap.add_argument("--iterations", type=int, default=2000)
    ap.add_argument("--out", default=None, help="also write E, P_fp64, P_mixed as text")
    ap.add_argument("--sweep", default=None, help="comma-separated J of a batched partial-wave gate")
    ap.add_argument("--cases-dir", default=None, help="where the generated input cases live (default: a temp dir)")
    ap.add_argument("--channels", action="store_true",
                    help="with --sweep: every reactant channel's max |dP_vj(E)| and max P_vj(E) per J")
    args = ap.parse_args()
    if args.sweep:
        print(json.dumps(run_sweep_gate(args.case, [int(x) for x in args.sweep.split(",")], args.iterations,
                                        cases_dir=args.cases_dir, channels=args.channels)))
        return
    out, e, a, b = run_gate(args.case, args.iterations, cases_dir=args.cases_dir)
    if args.out:
        np.savetxt(args.out, np.stack([e, a, b], 1), header="E(eV) P_fp64 P_mixed")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
