"""CPU oracle for the PencilFFTs transform path (test infrastructure only)."""
