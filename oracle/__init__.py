"""CPU oracle of the SPH hot path (test infrastructure only)."""
