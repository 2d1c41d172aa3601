"""CPU oracle for the vkhel hot path (test infrastructure only; see oracle.h)."""
