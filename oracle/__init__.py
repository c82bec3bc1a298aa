"""CPU oracle of the coupled thermal MRT-LBM step (test infrastructure only)."""
