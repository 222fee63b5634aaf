"""FP64 CPU oracle of the PHAFD hot path (test infrastructure only)."""
