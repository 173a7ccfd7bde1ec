"""Product-state projection for iprod = 2 (prodpaq / prodcvj,
SRC/mod_coortrans01_02.f:694-825), run on the device every iteration.

The tables are the ones the reference's ini_transcoor builds on the host
(mod_coortrans01_02.f:32-207: transRgjac, dtrans, prodwf, noBCprod); the
library takes them as given, in the C order of the Fortran arrays:

* ``transrgjac[ntot]`` on the wave's state vector layout,
* ``dtrans[ncan][nom][nang][n2p]`` = dtrans(n2prod0:n2prod1,
  nangproj0:nangproj1, iomminprod:iommaxprod, ncan),
* ``prodwf[nom][njp][nvp][nelec][nang][n2p]`` = prodwf(n2prod0:n2prod1,
  nangproj0:nangproj1, nelec, nviniprod:nvmaxprod, jiniprod:jmaxprod,
  iomminprod:iommaxprod),
* ``nobcprod[njp]`` = noBCprod(jiniprod:jmaxprod).

Results: zS2prod(E, v, j, Omega) as ``[nom][njp][nvp][netot]`` complex and the
last iteration's Cvjprod ``[nom][njp][nvp]``.
"""
from dataclasses import dataclass

import numpy as np


@dataclass
class ProductProjection:
    n2prod0: int
    n2prod1: int
    nangproj0: int
    nangproj1: int
    iomminprod: int
    iommaxprod: int
    jiniprod: int
    jmaxprod: int
    nviniprod: int
    nvmaxprod: int
    nobcprod: np.ndarray
    transrgjac: np.ndarray
    dtrans: np.ndarray
    prodwf: np.ndarray

    @property
    def shape(self):
        """(nom, njp, nvp) of Cvjprod."""
        return (self.iommaxprod - self.iomminprod + 1, self.jmaxprod - self.jiniprod + 1,
                self.nvmaxprod - self.nviniprod + 1)
