"""CPU oracle for the quantum-wire SBE path: test infrastructure only."""
