"""CPU oracle for the sw4lite time step (test infrastructure only)."""
