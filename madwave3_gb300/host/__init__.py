"""Host-side set-up of madwave3 runs (the modules the Fortran host keeps) and the
synthetic LEPS input generator."""
