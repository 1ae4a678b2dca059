"""CPU oracle package (test infrastructure)."""
