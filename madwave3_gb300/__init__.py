"""madwave3_gb300: GB300 (sm_103a) Chebyshev wave-packet propagator.

Drop-in for the H.psi application and Chebyshev loop of madwave3
(mod_Hphi_01y2, mod_absorcion_01y2, mod_flux_01y2, mod_PsiE_01y2 driven by
main_madwave3.f), behind the C-ABI in include/mw3gpu.h.

* :mod:`madwave3_gb300.host`   - the host-side set-up the Fortran program keeps
  (grid, basis, compressed potential, initial packet) and the synthetic input
  generator.
* :mod:`madwave3_gb300.propagator` - Python binding of the C-ABI.
* ``csrc/`` - the CUDA kernels and the C-ABI implementation (libmw3gpu.so).
"""
from .propagator import Mw3Error, Propagator, load_library  # noqa: F401
