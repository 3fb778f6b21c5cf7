"""CPU oracle for the msmpscu many-body force path (test infrastructure only)."""
