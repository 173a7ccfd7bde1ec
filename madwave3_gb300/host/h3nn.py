"""The neural-network H3 surface of the reference's H + HD example.

This is the potential ``pot.out`` tabulates for EXAMPLES/HD+H_collision
(EXAMPLES/HD+H_collision/pes/pothead.f: ``potelebond``;
EXAMPLES/HD+H_collision/pes/FFmodules.f90: ``NN_VH3`` and the routines it
calls), restated for numpy arrays of geometries.  The network takes the three
interatomic distances (bohr) through

* ``exponential``: e_i = exp(-alpha r_i), alpha = 0.7 (FFmodules.f90:285-294),
* ``fi_a3``: the permutation invariants p_1 = sum e_i, p_2 = sum e_i^2,
  p_3 = sum e_i^3 (:254-279),
* ``StandardScale``: (p - mean) / std (:296-306),
* two sigmoid layers of 20 and a linear output (``NN``, ``step``:
  :226-238, FFroutines.f:566-598),
* and rescales the output to hartree with the two ``ylinear`` numbers
  (:217-220).

The weights are single-precision literals of Fortran data statements, so
their values are the float32 numbers widened to double; the constant alpha
is such a literal too (``7e-1``).  They are read from a JSON file of their
decimal text (``tests/golden/h3nn_weights.json``, extracted from
FFmodules.f90), since this surface is an input of the example, not part of
the propagator.

``potelebond`` (pothead.f:26-55) refers the energy to H2 at r = 1.4 bohr with
the third atom at 100 bohr, computes the third distance from (r1, r2,
cos theta) and clamps every distance at 0.25 bohr.
"""
import json
import re

import numpy as np

ALPHA = float(np.float32(0.7))       # the single-precision literal 7e-1


def _f32(text):
    return float(np.float32(text))


def _fill(arr, spec, vals):
    """One data statement: ``idx`` like '1,1:5', '3,:', ':' or '7' (1-based)."""
    parts = spec.split(",")
    sl = []
    for k, p in enumerate(parts):
        if p == ":":
            sl.append(slice(None))
        elif ":" in p:
            a, b = p.split(":")
            sl.append(slice(int(a) - 1, int(b)))
        else:
            sl.append(int(p) - 1)
    view = arr[tuple(sl)]
    flat = np.array([_f32(v) for v in vals])
    if np.ndim(view) == 0:
        arr[tuple(sl)] = flat[0]
    else:
        arr[tuple(sl)] = flat.reshape(np.shape(view))


class H3NN:
    """Vectorised NN_VH3 / potelebond of the example's H3 surface."""

    def __init__(self, weights):
        if isinstance(weights, str):
            with open(weights) as f:
                weights = json.load(f)
        n1, n2, n3, n4 = weights["n"]
        shapes = {"xstandard": (n1, 2), "ylinear": (2,), "w": (n1, n2), "b": (n2,), "w1": (n2, n3),
                  "b1": (n3,), "w2": (n3, n4), "b2": (n4,)}
        self.a = {k: np.zeros(s) for k, s in shapes.items()}
        for name, stmts in weights["arrays"].items():
            for spec, vals in stmts:
                _fill(self.a[name], re.sub(r"\s", "", spec), vals)
        r = np.array([100.0]), np.array([100.0]), np.array([1.4])
        self.vref = float(self.vh3(*r)[0])

    def vh3(self, ra, rb, rc):
        """NN_VH3: energy (hartree) of the three distances (bohr), any shape."""
        a = self.a
        shape = np.shape(ra)
        d = [np.ravel(np.asarray(x, np.float64)) for x in (ra, rb, rc)]
        e = [np.exp(-ALPHA * x) for x in d]
        p = np.stack([e[0] + e[1] + e[2],
                      e[0] * e[0] + e[1] * e[1] + e[2] * e[2],
                      e[0] * e[0] * e[0] + e[1] * e[1] * e[1] + e[2] * e[2] * e[2]], 1)
        x = (p - a["xstandard"][:, 0]) / a["xstandard"][:, 1]
        h = self._layer(x, a["w"], a["b"], True)
        h = self._layer(h, a["w1"], a["b1"], True)
        out = self._layer(h, a["w2"], a["b2"], False)[:, 0]
        y1, y2 = a["ylinear"]
        return (0.5 * (out + 1.0) * (y1 - y2) + y2).reshape(shape)

    @staticmethod
    def _layer(x, w, b, sigmoid):
        # step (FFroutines.f:566-598): b(i) + sum_j x(j) w(j,i), summed in j order
        o = np.broadcast_to(b, (x.shape[0], b.size)).copy()
        for j in range(w.shape[0]):
            o = o + x[:, j:j + 1] * w[j][None, :]
        if sigmoid:
            o = 1.0 / (1.0 + np.exp(-o))
        return o

    def potelebond(self, r1, r2, costet):
        """pothead.f:26-55: V(r1, r2, cos theta) - V_ref in hartree, as a
        [1][1][...] diabatic matrix (one electronic state)."""
        r1 = np.asarray(r1, np.float64)
        r2 = np.asarray(r2, np.float64)
        r3 = np.sqrt(r1 * r1 + r2 * r2 - 2.0 * r1 * r2 * costet)
        r1 = np.maximum(r1, 0.25)
        r2 = np.maximum(r2, 0.25)
        r3 = np.maximum(r3, 0.25)
        v = self.vh3(r3, r2, r1) - self.vref
        return v[None, None]
