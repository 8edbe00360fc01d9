"""CPU oracle for the EP training path (test infrastructure only)."""
