"""CPU oracle of the MPM substep (test infrastructure; see mpm_oracle.c)."""
