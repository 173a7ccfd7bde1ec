"""Physical constants and unit conventions of madwave3 ("zots").

Energies are carried in zots (E[zot] = E[cm^-1] * conve1), lengths in
angstrom and masses in amu, exactly as the Fortran host does
(SRC/mod_gridYpara_01y2.f:13-31).  The values below are the reference's
parameters; they have to be the same numbers for the propagation to be
identical.
"""
import math

pi = math.acos(-1.0)
conve1 = 1.197e-4            # cm^-1 -> zot
convl = 0.52917726           # bohr -> angstrom
convm = 0.182288853e4        # amu -> electron masses
conve = 4.55633538e-6        # cm^-1 -> hartree
eV2cm = 8065.5
hbr = convl / math.sqrt(convm * conve / conve1)
au2eV = 27.21113957
zot2au = 0.0380646230576441
zot2eV = 1.03578177070099
hartree2cm = 219474.625


def ev_to_zot(e_ev):
    """eV -> zot, as the reference converts namelist energies (ev2cm*conve1)."""
    return e_ev * eV2cm * conve1


def zot_to_ev(e_zot):
    return e_zot / conve1 / eV2cm
