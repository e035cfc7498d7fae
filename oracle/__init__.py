"""CPU oracle for the LGT exact-diagonalisation path (test infrastructure only)."""
