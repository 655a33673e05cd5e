"""FP64 CPU oracle of the TCSEM_FDTD time-stepping path (test infrastructure only)."""
