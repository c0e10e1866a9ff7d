"""CPU oracle for the LACE preconditioned-solve path (test infrastructure only)."""
