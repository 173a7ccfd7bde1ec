"""Reduced Wigner rotation matrices and Gauss-Legendre quadrature.

These are the two numerical routines of the reference's angular set-up that
the host side keeps (mod_gridYpara / mod_baseYfunciones are not part of the
GPU path, but their tables feed it).  The algorithms are the published ones
the reference uses, restated here:

* ``gauleg`` - Gauss-Legendre nodes/weights by Newton iteration on P_n with
  the starting guess cos(pi (i-1/4)/(n+1/2)), nodes ordered from -1 to +1
  (SRC/liboctdyn.f:174-211).
* ``dwigner`` - d^j_{m,m'}(beta) for j = jmin..jmax by the three-term upward
  recursion in j started from the closed form at j = max(|m|,|m'|)
  (SRC/liboctdyn.f:3-171).  Half-integer j are indexed by 2j as in the
  reference.
"""
import math

import numpy as np


def gauleg(n):
    """Return (weights, nodes) of the n-point Gauss-Legendre rule on [-1,1]."""
    w = np.zeros(n)
    x = np.zeros(n)
    yn = float(n)
    eps = 1.0e-15
    m = (n + 1) // 2
    xm, xl = 0.0, 1.0
    for i in range(1, m + 1):
        z = math.cos(math.pi * (i - 0.25) / (yn + 0.5))
        while True:
            p1, p2 = 1.0, 0.0
            for j in range(1, n + 1):
                p3 = p2
                p2 = p1
                p1 = ((2.0 * j - 1.0) * z * p2 - (j - 1.0) * p3) / j
            pp = yn * (z * p1 - p2) / (z * z - 1.0)
            z1 = z
            z = z1 - p1 / pp
            if abs(z - z1) <= eps:
                break
        x[i - 1] = xm - xl * z
        x[n - i] = xm + xl * z
        w[i - 1] = 2.0 * xl / ((1.0 - z * z) * pp * pp)
        w[n - i] = w[i - 1]
    return w, x


def dwigner(jmax2, m2, mp2, beta, ndim=None):
    """d^J_{M,M'}(beta) stored at index 2J, for 2J = 0..jmax2.

    m2, mp2 are 2M and 2M'.  Entries below J = max(|M|,|M'|) are zero.
    Raises on the complex-phase case the reference stops on.
    """
    n = jmax2 if ndim is None else ndim
    dj = np.zeros(n + 1)
    jmin2 = max(abs(m2), abs(mp2))
    y = math.cos(beta)
    if jmin2 == 0:
        dj[0] = 1.0
        if jmax2 >= 2:
            dj[2] = y
        for ind in range(4, jmax2 + 1, 2):
            xj = ind * 0.5
            dj[ind] = (y * (2.0 * xj - 1.0) * dj[ind - 2] - (xj - 1.0) * dj[ind - 4]) / xj
        return dj
    # closed form at J = jmin
    facnum = sum(math.log(float(i)) for i in range(1, jmin2 + 1))
    mreal2 = mp2 if jmin2 == abs(m2) else m2
    facden1 = sum(math.log(i * 0.5) for i in range(2, jmin2 + mreal2 + 1, 2)) if jmin2 + mreal2 > 0 else 0.0
    facden2 = sum(math.log(i * 0.5) for i in range(2, jmin2 - mreal2 + 1, 2)) if jmin2 - mreal2 > 0 else 0.0
    fact = math.exp(0.5 * (facnum - facden1 - facden2))
    sign = 1.0
    xsin = math.sin(beta * 0.5)
    xcos = math.cos(beta * 0.5)
    a = b = 0.0
    if jmin2 == abs(m2):
        if jmin2 == m2:
            if (jmin2 - mp2) % 2 == 0:
                sign = float((-1) ** int((jmin2 - mp2) * 0.5 + 0.5))
                a = xsin ** ((jmin2 - mp2) * 0.5)
                b = xcos ** ((jmin2 + mp2) * 0.5)
            else:
                raise ValueError("dwigner: complex phase")
        elif jmin2 == -m2:
            a = xsin ** ((jmin2 + mp2) * 0.5)
            b = xcos ** ((jmin2 - mp2) * 0.5)
    elif jmin2 == abs(mp2):
        if jmin2 == mp2:
            a = xsin ** ((jmin2 - m2) * 0.5)
            b = xcos ** ((jmin2 + m2) * 0.5)
        elif jmin2 == -mp2:
            if (jmin2 + m2) % 2 == 0:
                sign = float((-1) ** int((jmin2 + m2) * 0.5 + 0.5))
                a = xsin ** ((jmin2 + m2) * 0.5)
                b = xcos ** ((jmin2 - m2) * 0.5)
            else:
                raise ValueError("dwigner: complex phase")
    dj[jmin2] = fact * sign * a * b
    # J = jmin + 1
    xj = jmin2 * 0.5
    xjp = xj + 1.0
    xm = m2 * 0.5
    xmp = mp2 * 0.5
    facnum = xjp * (2.0 * xj + 1.0)
    facden1 = xjp * xjp - xm * xm
    facden2 = xjp * xjp - xmp * xmp
    factot = facnum / math.sqrt(facden1 * facden2)
    facj = y - xm * xmp / (xj * (xj + 1.0))
    if jmin2 + 2 <= jmax2:
        dj[jmin2 + 2] = factot * facj * dj[jmin2]
        for indp in range(jmin2 + 4, jmax2 + 1, 2):
            ind = indp - 2
            indm = indp - 4
            xjp = indp * 0.5
            xj = xjp - 1.0
            facnum = xjp * (2.0 * xj + 1.0)
            facden1 = xjp * xjp - xm * xm
            facden2 = xjp * xjp - xmp * xmp
            factot = facnum / math.sqrt(facden1 * facden2)
            facj = y - xm * xmp / (xj * (xj + 1.0))
            fac1jm = xj * xj - xm * xm
            fac2jm = xj * xj - xmp * xmp
            facden = xj * (2.0 * xj + 1.0)
            facjm = math.sqrt(fac1jm * fac2jm) / facden
            dj[indp] = factot * (facj * dj[ind] - facjm * dj[indm])
    return dj


def dwigner_vec(jmax2, m2, mp2, beta):
    """dwigner for an array of angles at once: returns [len(beta), jmax2+1]."""
    beta = np.asarray(beta, dtype=np.float64)
    nb = beta.shape[0]
    dj = np.zeros((nb, jmax2 + 1))
    jmin2 = max(abs(m2), abs(mp2))
    y = np.cos(beta)
    if jmin2 == 0:
        dj[:, 0] = 1.0
        if jmax2 >= 2:
            dj[:, 2] = y
        for ind in range(4, jmax2 + 1, 2):
            xj = ind * 0.5
            dj[:, ind] = (y * (2.0 * xj - 1.0) * dj[:, ind - 2] - (xj - 1.0) * dj[:, ind - 4]) / xj
        return dj
    facnum = sum(math.log(float(i)) for i in range(1, jmin2 + 1))
    mreal2 = mp2 if jmin2 == abs(m2) else m2
    facden1 = sum(math.log(i * 0.5) for i in range(2, jmin2 + mreal2 + 1, 2)) if jmin2 + mreal2 > 0 else 0.0
    facden2 = sum(math.log(i * 0.5) for i in range(2, jmin2 - mreal2 + 1, 2)) if jmin2 - mreal2 > 0 else 0.0
    fact = math.exp(0.5 * (facnum - facden1 - facden2))
    sign = 1.0
    xsin = np.sin(beta * 0.5)
    xcos = np.cos(beta * 0.5)
    if jmin2 == abs(m2):
        if jmin2 == m2:
            if (jmin2 - mp2) % 2 != 0:
                raise ValueError("dwigner: complex phase")
            sign = float((-1) ** int((jmin2 - mp2) * 0.5 + 0.5))
            a = xsin ** ((jmin2 - mp2) * 0.5)
            b = xcos ** ((jmin2 + mp2) * 0.5)
        else:
            a = xsin ** ((jmin2 + mp2) * 0.5)
            b = xcos ** ((jmin2 - mp2) * 0.5)
    else:
        if jmin2 == mp2:
            a = xsin ** ((jmin2 - m2) * 0.5)
            b = xcos ** ((jmin2 + m2) * 0.5)
        else:
            if (jmin2 + m2) % 2 != 0:
                raise ValueError("dwigner: complex phase")
            sign = float((-1) ** int((jmin2 + m2) * 0.5 + 0.5))
            a = xsin ** ((jmin2 + m2) * 0.5)
            b = xcos ** ((jmin2 - m2) * 0.5)
    dj[:, jmin2] = fact * sign * a * b
    xj = jmin2 * 0.5
    xm = m2 * 0.5
    xmp = mp2 * 0.5
    xjp = xj + 1.0
    factot = xjp * (2.0 * xj + 1.0) / math.sqrt((xjp * xjp - xm * xm) * (xjp * xjp - xmp * xmp))
    facj = y - xm * xmp / (xj * (xj + 1.0))
    if jmin2 + 2 <= jmax2:
        dj[:, jmin2 + 2] = factot * facj * dj[:, jmin2]
        for indp in range(jmin2 + 4, jmax2 + 1, 2):
            xjp = indp * 0.5
            xj = xjp - 1.0
            factot = xjp * (2.0 * xj + 1.0) / math.sqrt((xjp * xjp - xm * xm) * (xjp * xjp - xmp * xmp))
            facj = y - xm * xmp / (xj * (xj + 1.0))
            facjm = math.sqrt((xj * xj - xm * xm) * (xj * xj - xmp * xmp)) / (xj * (2.0 * xj + 1.0))
            dj[:, indp] = factot * (facj * dj[:, indp - 2] - facjm * dj[:, indp - 4])
    return dj
