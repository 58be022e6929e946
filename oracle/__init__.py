"""CPU oracle for the GENFIRE hot path (test infrastructure only)."""
