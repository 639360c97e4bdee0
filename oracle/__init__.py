"""CPU oracle of the finite-difference hot path (test infrastructure only)."""
