"""CPU oracle for the SPH step (test infrastructure only)."""
