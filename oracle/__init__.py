"""CPU oracle of the PBSM3D step (test infrastructure only)."""
