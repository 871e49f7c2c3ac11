"""CPU oracle for the Nixis hot path (test infrastructure only)."""
