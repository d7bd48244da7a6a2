"""CPU oracle for the local-neighborhood operator (test infrastructure only)."""
