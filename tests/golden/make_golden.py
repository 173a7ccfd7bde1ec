"""Extract the golden numbers the oracle and the GPU path are pinned against
from the reference's own example files, into tests/golden/.

Run once in a checkout where the reference is available:

    python tests/golden/make_golden.py /path/to/madwave3

Sources (inside the reference):

* EXAMPLES/HD+H_collision/J000-check/sal.000, the log of the shipped J=0 run:
  its namelists, Gauss-Legendre angles, absorber start, kinetic energy range,
  collision packet, flux line, energy interval and the energy-domain norm of
  the packet (reference_pins.json); and the numbers that depend on the
  example's neural-network H3 surface (example_pins.json): the reactant and
  product diatomic energies, the stored points per process, the initial
  packet's norm and mean energy and the norm trace ||psi_k||^2, k = 1..4001;
* J000-check/S2prod.v00.J000.k00008, the same run's probability file
  (its layout in reference_pins.json, every row in example_pins.json);
* EXAMPLES/HD+H_collision/README.md (the 60-angle list of its pot.out run);
* EXAMPLES/HD+H_collision/input.dat, the run's namelists (example_pins.json);
* EXAMPLES/HD+H_collision/pes/FFmodules.f90: the weights and scalings of the
  example's neural-network surface, kept as their decimal text (h3nn_weights.json).
"""
import json
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def floats(line):
    return [float(x.replace("D", "E")) for x in re.findall(r"-?\d+\.\d*(?:[EeDd][-+]?\d+)?", line)]


def reference_pins(ref, sal):
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
    return out, s2p


def _table_after(sal, header, ncols):
    """Rows of ncols numbers (leading integer columns) after the header line, up
    to the first line that is not such a row."""
    i0 = next(i for i, l in enumerate(sal) if l.strip().startswith(header))
    rows = []
    started = False
    for l in sal[i0 + 1:]:
        t = l.split()
        if len(t) == ncols and all(re.fullmatch(r"-?\d+", x) for x in t[:-1]):
            rows.append([int(x) for x in t[:-1]] + [float(t[-1].replace("D", "E"))])
            started = True
        elif started:
            break
    return rows


def example_pins(ref, sal, s2p):
    """The numbers of the shipped run that depend on its neural-network surface,
    and the run's input file."""
    out = {"source": "EXAMPLES/HD+H_collision/J000-check/sal.000 and S2prod.v00.J000.k00008",
           "input_dat": open(os.path.join(ref, "EXAMPLES/HD+H_collision/input.dat")).read()}
    # reactant (01) diatomic levels minus ediatref: ie, j, v, E(eV)
    out["reactant_levels_ev"] = _table_after(sal, "ie  j   v   E(eV)", 4)
    # product (02) diatomic levels minus ediatref: j, v, E(eV)
    out["product_levels_ev"] = _table_after(sal, "j   v   E(eV)", 3)
    out["ntotproc"] = [int(l.split("=")[1]) for l in sal if "ntotproc=" in l and "in processor" in l]
    for l in sal:
        if "Vmin(eV)=" in l and "E_kin" not in l:
            out["vmin_ev"] = floats(l)[-1]
        if "** Norm of initial wavepacket=" in l:
            out["initial_norm"] = floats(l)[-1]
        if "Mean energy (eV) and norm of initial wvp=" in l:
            out["mean_energy_ev"] = floats(l)[-1]
        if "initial norm proc=" in l:
            out.setdefault("initial_norm_proc", []).append(floats(l)[-1])
        if "nfluxproc=" in l:
            out["nfluxproc_rank0"] = int(l.split("=")[-1])
    norms = {}
    i0 = next(i for i, l in enumerate(sal) if "k            norm" in l)
    for l in sal[i0 + 1:]:
        t = l.split()
        if len(t) == 2 and t[0].isdigit():
            norms[int(t[0])] = float(t[1].replace("D", "E"))
    ks = sorted(norms)
    assert ks == list(range(1, len(ks) + 1)), "gap in the norm trace"
    out["norm_trace"] = [norms[k] for k in ks]
    out["product_wf_norms"] = [[int(a), int(b), int(c), float(d)] for a, b, c, d in
                               re.findall(r"norm \(iom,j,v=\s*(\d+),\s*(\d+),\s*(\d+)\s*\)=\s*(\S+)", "\n".join(sal))]
    out["s2prod_rows"] = [[float(x) for x in l.split()] for l in s2p if l.strip()]
    return out


def nn_weights(ref):
    """The data statements of the example's neural-network surface, as text."""
    src = open(os.path.join(ref, "EXAMPLES/HD+H_collision/pes/FFmodules.f90")).read()
    shapes = {}
    for m in re.finditer(r"integer, parameter, private :: (.*)", src):
        for name, val in re.findall(r"(\w+)\s*=\s*(\d+)", m.group(1)):
            shapes[name] = int(val)
    out = {"source": "EXAMPLES/HD+H_collision/pes/FFmodules.f90",
           "note": "single-precision literals of Fortran data statements (kept as text)",
           "n": [shapes["n1"], shapes["n2"], shapes["n3"], shapes["n4"]], "arrays": {}}
    for name, idx, vals in re.findall(r"^data\s+(\w+)\(([^)]*)\)\s*/([^/]*)/", src, re.M):
        out["arrays"].setdefault(name, []).append([idx.replace(" ", ""), [v.strip() for v in vals.split(",")]])
    return out


def main(ref):
    sal = open(os.path.join(ref, "EXAMPLES/HD+H_collision/J000-check/sal.000")).read().splitlines()
    pins, s2p = reference_pins(ref, sal)
    with open(os.path.join(HERE, "reference_pins.json"), "w") as f:
        json.dump(pins, f, indent=1)
    with open(os.path.join(HERE, "example_pins.json"), "w") as f:
        json.dump(example_pins(ref, sal, s2p), f, separators=(",", ":"))
    with open(os.path.join(HERE, "h3nn_weights.json"), "w") as f:
        json.dump(nn_weights(ref), f, indent=0)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py REFERENCE_CHECKOUT")
    main(sys.argv[1])
