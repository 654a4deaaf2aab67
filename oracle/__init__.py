"""CPU oracle of the BSAM 1.2 FAS V-cycle (test infrastructure only)."""
