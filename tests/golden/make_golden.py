"""Extract the golden numbers the oracle is pinned against from the
reference's own example files, into tests/golden/reference_pins.json.

Run once in a checkout where the reference is available:

    python tests/golden/make_golden.py /path/to/madwave3

Sources (inside the reference): EXAMPLES/HD+H_collision/J000-check/sal.000
(the log of the shipped J=0 run: its namelists, Gauss-Legendre angles,
absorber start, kinetic energy range, collision packet, flux line, energy
interval and the energy-domain norm of the packet), the layout and first
lines of the same run's S2prod.v00.J000.k00008, and
EXAMPLES/HD+H_collision/README.md (the 60-angle list of its pot.out run).
Only numbers that do not depend on the example's neural-network PES are kept.
"""
import json
import os
import re
import sys


def floats(line):
    return [float(x.replace("D", "E")) for x in re.findall(r"-?\d+\.\d*(?:[EeDd][-+]?\d+)?", line)]


def main(ref):
    sal = open(os.path.join(ref, "EXAMPLES/HD+H_collision/J000-check/sal.000")).read().splitlines()
    out = {"source": "EXAMPLES/HD+H_collision/J000-check/sal.000, EXAMPLES/HD+H_collision/README.md"}
    # namelist values echoed in the log
    nml = {}
    for line in sal:
        m = re.match(r"\s*([A-Z0-9_]+)=\s*\"?([^,\"]+)\"?\s*,", line)
        if m:
            nml.setdefault(m.group(1).lower(), m.group(2).strip())
    out["namelist"] = nml
    # Gauss-Legendre angles (degrees), iang 1..140
    i0 = next(i for i, l in enumerate(sal) if "Angular grid to plot" in l)
    ang = []
    for l in sal[i0 + 1:]:
        t = l.split()
        if len(t) == 2 and t[0].isdigit():
            ang.append(float(t[1]))
            if len(ang) == int(nml["nangu"]):
                break
    out["angles_deg_140"] = ang
    for l in sal:
        if "Absorption starts at ir1,ir2" in l:
            out["ir1abs_ir2abs"] = [int(x) for x in l.split("=")[1].split()]
        if "E_kin^1(max)=" in l:
            out["ekin1max_ev"], out["ekin2max_ev"] = floats(l)[-2:] if len(floats(l)) >= 2 else floats(l)
        if "E_kin^1(min)=" in l:
            v = floats(l)
            out["ekin1min_ev"], out["ekin2min_ev"] = v[-2], v[-1]
        if "r20 =" in l:
            v = floats(l)
            out["r20"], out["k0"], out["alpha0"] = v[0], v[1], v[2]
        if "norm of incident gaussian in R2=" in l:
            out["gauss_norm"] = floats(l)[-1]
        if "total flux evaluated at index ir4flux=" in l:
            out["ir4flux"] = int(l.split("=")[1])
        if "Emin=" in l and "Emax=" in l:
            v = floats(l)
            out["emin_ev"], out["emax_ev"] = v[0], v[1]
        if "Norm ini. wvp in energy=" in l:
            out["norm_in_energy"] = floats(l)[-1]
    readme = open(os.path.join(ref, "EXAMPLES/HD+H_collision/README.md")).read().splitlines()
    i0 = next(i for i, l in enumerate(readme) if "Angular grid to plot" in l)
    a60 = []
    for l in readme[i0 + 1:]:
        t = l.split()
        if len(t) == 2 and t[0].isdigit():
            a60.append([int(t[0]), float(t[1])])
        elif a60 and "..." in l:
            break
    out["angles_deg_60_head"] = a60
    # the shipped run's S2prod file (iprod = 2): its layout and first lines, for
    # the format of the probability files the post-processing programs read
    s2p = open(os.path.join(ref, "EXAMPLES/HD+H_collision/J000-check/S2prod.v00.J000.k00008")).read().splitlines()
    out["s2prod"] = {"file": "EXAMPLES/HD+H_collision/J000-check/S2prod.v00.J000.k00008",
                     "lines": len(s2p), "columns": len(s2p[0].split()), "head": s2p[:3], "tail": s2p[-1:]}
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_pins.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
